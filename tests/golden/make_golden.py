"""Generates the golden fixtures in tests/golden/ from the HODLR3D reference.

The reference's own sources are compiled (oracle/Makefile.ref, against the
project-written Eigen/Boost API shim in oracle/shim) into
oracle/_ref/hodlr3d_ref, which is run on each case below; its dumps are
canonicalised and stored as compressed .npz files.  Only needed where the
reference checkout is present; the fixtures themselves are committed.

    python tests/golden/make_golden.py --ref <reference checkout> [--only NAME]

(or HODLR3D_REFERENCE=<reference checkout> in the environment).  Each case is
also run through oracle/_ref/hodlr3d_ref_plain, the same sources with plain
left-to-right norms and dot products in the shim, and the number of blocks
whose ACA rank differs between the two reduction orders is stored
(rank_flips_plain_sums): it says how much "identical ranks" depends on the
shim's canonical reduction order at the Eigen boundary.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from hodlr3d_gb300 import workloads  # noqa: E402

# name -> (points generator, args, nP1D, L, TOL_POW, Qchoice, diag, gmres maxit, full pivots)
CASES = {
    # 16^3 cell centres, leaf 64, depth 2, 1/r with quadrature diagonal, tol 1e-10
    "grid16_q16_tol10": ("grid_cell_centres", (16,), 4, 1.0, 10, 16, "nan", 50, True),
    # 4096 uniform random points, Poisson leaves, tol 1e-12
    "rand4096_q16_tol12": ("uniform_random", (4096, 1), 4, 1.0, 12, 16, "nan", 50, True),
    # the reference's benchmark settings: interior nodes, 20^3, leaf 5^3, 1/r, tol 1e-7
    "refnodes20_q7_tol7": ("grid_reference_nodes", (20,), 6, 1.0, 7, 7, "nan", 0, True),
    # exp(-r) with diagonal 1, tol 1e-8
    "grid16_q1diag1_tol8": ("grid_cell_centres", (16,), 4, 1.0, 8, 1, "1.0", 30, True),
    # depth 3 with leaves of 8 points
    "grid16_leaf8_q16_tol10": ("grid_cell_centres", (16,), 2, 1.0, 10, 16, "nan", 0, False),
    # depth 3 with leaves of 64 points (32768 points); the deeper cases store the
    # pivots as one hash per target box
    "grid32_q16_tol10": ("grid_cell_centres", (32,), 4, 1.0, 10, 16, "nan", 0, False),
    # depth 4 with one point per leaf, domain half-width 2
    "grid16_leaf1_q4_tol8": ("grid_cell_centres", (16, 2.0), 1, 2.0, 8, 4, "nan", 0, False),
    # the Bessel-function kernels: J0(r), Y0(r), K_{1/2}(r)/sqrt(r)
    "grid16_q11_tol8": ("grid_cell_centres", (16,), 4, 1.0, 8, 11, "nan", 0, True),
    "grid16_q12_tol8": ("grid_cell_centres", (16,), 4, 1.0, 8, 12, "nan", 0, True),
    "grid16_q14_tol8": ("grid_cell_centres", (16,), 4, 1.0, 8, 14, "nan", 0, True),
    # 32^3 grid at tol 1e-12 and 32768 uniform random points at tol 1e-12: the
    # plain FP64 form at scale
    "grid32_q16_tol12": ("grid_cell_centres", (32,), 4, 1.0, 12, 16, "nan", 0, False),
    "rand32768_q16_tol12": ("uniform_random", (32768, 1), 4, 1.0, 12, 16, "nan", 0, False),
    # 64^3 grid (depth 4, 262144 points), 1/r with quadrature diagonal, tol 1e-10:
    # the operator of the solve/adjoint workload and of the batched-product benchmark
    "grid64_q16_tol10": ("grid_cell_centres", (64,), 4, 1.0, 10, 16, "nan", 40, False),
    # 64^3 grid, exp(-r) with diagonal 1, tol 1e-8: the precision/batching workload
    "grid64_q1diag1_tol8": ("grid_cell_centres", (64,), 4, 1.0, 8, 1, "1.0", 0, False),
}


def points_hash(pts: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(pts, np.float64).tobytes()).hexdigest()


def pivot_hash(rows: np.ndarray, cols: np.ndarray) -> int:
    return zlib.crc32(np.ascontiguousarray(np.stack([rows, cols]), np.int32).tobytes())


def run_case(binary: str, name: str, spec, ranks_only: bool = False) -> dict:
    gen, args, nP1D, L, tol, q, diag, gmres_maxit, full_piv = spec
    if ranks_only:
        gmres_maxit = 0
    pts = getattr(workloads, gen)(*args)
    N = len(pts)
    charges = workloads.charges_uniform(N, seed=1)
    with tempfile.TemporaryDirectory() as td:
        ind, outd = os.path.join(td, "in"), os.path.join(td, "out")
        os.makedirs(ind)
        os.makedirs(outd)
        pts.astype("<f8").tofile(os.path.join(ind, "points.f64"))
        charges.astype("<f8").tofile(os.path.join(ind, "charges.f64"))
        cmd = [binary, ind, outd, str(nP1D), str(L), str(tol), str(q), diag, str(gmres_maxit), "1e-10"]
        print(name, ":", subprocess.run(cmd, check=True, capture_output=True, text=True).stdout.strip())

        def rd(fn, dt):
            return np.fromfile(os.path.join(outd, fn), dt)

        N_, levels = rd("meta.i32", np.int32)
        assert N_ == N
        lv, bx, src = rd("il_level.i32", np.int32), rd("il_box.i32", np.int32), rd("il_idx.i32", np.int32)
        rank = rd("rank.i32", np.int32)
        if ranks_only:
            keep = lv >= 1
            order = np.lexsort((src[keep], bx[keep], lv[keep]))
            return dict(rank=rank[np.nonzero(keep)[0][order]])
        pp = rd("piv_ptr.i32", np.int32)
        rp, cp = rd("row_piv.i32", np.int32), rd("col_piv.i32", np.int32)
        keep = lv >= 1
        order = np.lexsort((src[keep], bx[keep], lv[keep]))
        idx = np.nonzero(keep)[0][order]
        pairs = np.stack([lv[idx], bx[idx], src[idx]], axis=1).astype(np.int32)
        out = dict(
            name=np.array(name), generator=np.array(gen), gen_args=np.array(args, dtype=np.float64),
            points_sha256=np.array(points_hash(pts)), nP1D=np.int32(nP1D), L=np.float64(L),
            tol_pow=np.int32(tol), kernel=np.int32(q), diag=np.float64(float(diag)),
            N=np.int64(N), levels=np.int32(levels), kii=rd("kii.f64", np.float64),
            perm=rd("perm.i32", np.int32), leaf_count=rd("leaf_count.i32", np.int32),
            centers=rd("centers.f64", np.float64),
            nbr=rd("nbr.i32", np.int32).astype(np.int16 if levels <= 5 else np.int32),
            rank=rank[idx].astype(np.int16),
            matvec=rd("matvec.f64", np.float64),
            stats=rd("stats.f64", np.float64),
        )
        out["pair_count_per_level"] = np.bincount(pairs[:, 0], minlength=levels + 1).astype(np.int64)
        if len(pairs) <= 20000:
            out["pairs"] = pairs.astype(np.int16)
        out["pairs_sha256"] = np.array(hashlib.sha256(pairs.tobytes()).hexdigest())
        if full_piv:
            rows = np.concatenate([rp[pp[i]:pp[i + 1]] for i in idx]) if len(idx) else np.zeros(0, np.int32)
            cols = np.concatenate([cp[pp[i]:pp[i + 1]] for i in idx]) if len(idx) else np.zeros(0, np.int32)
            out["row_piv"] = rows.astype(np.int16 if N < 32768 else np.int32)
            out["col_piv"] = cols.astype(np.int16 if N < 32768 else np.int32)
        else:
            # one CRC32 per target box (level, box) over its pairs' pivots in
            # canonical order; idx is sorted by (level, box, source), so every
            # box is one run of it
            key = pairs[:, 0].astype(np.int64) * (1 << 32) + pairs[:, 1]
            starts = np.concatenate([[0], np.nonzero(np.diff(key))[0] + 1, [len(key)]])
            crcs = []
            for a, b in zip(starts[:-1], starts[1:]):
                sel = idx[a:b]
                rows = np.concatenate([rp[pp[i]:pp[i + 1]] for i in sel])
                cols = np.concatenate([cp[pp[i]:pp[i + 1]] for i in sel])
                crcs.append(pivot_hash(rows, cols))
            out["piv_crc_box"] = np.array(crcs, dtype=np.uint32)
        if gmres_maxit > 0:
            out["gmres_hist"] = rd("gmres_hist.f64", np.float64)
            out["gmres_nit"] = rd("gmres_nit.i32", np.int32)
            out["gmres_maxit"] = np.int32(gmres_maxit)
            out["gmres_x"] = rd("gmres_x.f64", np.float64)
        out["ref_times"] = rd("times.f64", np.float64)
        return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("HODLR3D_REFERENCE"))
    ap.add_argument("--only", default=None, help="comma-separated case names")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref <reference checkout> or set HODLR3D_REFERENCE")
    subprocess.run(["make", "-s", "-j8", "-f", "oracle/Makefile.ref", f"REF={a.ref}"], cwd=ROOT, check=True)
    binary = os.path.join(ROOT, "oracle", "_ref", "hodlr3d_ref")
    plain = os.path.join(ROOT, "oracle", "_ref", "hodlr3d_ref_plain")
    only = set(a.only.split(",")) if a.only else None
    for name, spec in CASES.items():
        if only and name not in only:
            continue
        data = run_case(binary, name, spec)
        alt = run_case(plain, name + " (plain sums)", spec, ranks_only=True)
        data["rank_flips_plain_sums"] = np.int64(np.count_nonzero(alt["rank"] != data["rank"]))
        print(name, ": blocks whose rank changes with plain sums:", int(data["rank_flips_plain_sums"]))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)


if __name__ == "__main__":
    main()
