"""A fixed workload for external profilers (ncu): assemble the operator on a
grid of cell centres, then run each requested product once, in order.

    python -m hodlr3d_gb300.profile_run --n 32 --nrhs 1 --precisions mixed fp64x --transpose

For every precision: A x, then (with --transpose) A^T x.  Prints one line
with the operator's size when done; nothing is timed here (bench.py times).
"""
from __future__ import annotations

import argparse


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=32, help="grid points per axis")
    ap.add_argument("--nrhs", type=int, default=1)
    ap.add_argument("--tol-pow", type=int, default=10)
    ap.add_argument("--qchoice", type=int, default=16)
    ap.add_argument("--precisions", nargs="+", default=["mixed"], choices=["fp64", "mixed", "fp64x"])
    ap.add_argument("--transpose", action="store_true")
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args()
    import torch

    from . import HODLR3D
    from .workloads import charges_normal, grid_cell_centres
    H = HODLR3D(4, 1.0, a.tol_pow, a.qchoice, grid_cell_centres(a.n))
    H.assemble()
    X = torch.tensor(charges_normal(H.N, a.nrhs, seed=11), device="cuda").reshape(H.N, a.nrhs)
    for _ in range(a.repeat):
        for prec in a.precisions:
            H.matvec(X, prec)
            if a.transpose:
                H.matvec(X, prec, transpose=True)
    torch.cuda.synchronize()
    H.device_status()
    st = H.stats()
    print(f"n={H.N} pairs={st['n_pairs']} factor_entries={st['factor_entries']}")
    H.close()


if __name__ == "__main__":
    main()
