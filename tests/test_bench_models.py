"""bench.py's work models, on the CPU: the ACA work at the produced ranks
(assembly roofline) against a hand count, and the per-engine algorithmic bytes
of the matvec kernels (matvec roofline): every span name an engine's CUDA
source marks has a byte count under that engine, and on the 16^3 golden tree
the factor bytes of each engine add up to the factor entries of the ranks."""
import os
import re
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
import golden_util as gu  # noqa: E402

SOURCES = {"simt": "matvec.cu", "tc": "matvec_tc.cu", "gemv": "matvec_gemv.cu", "f64": "matvec_f64.cu"}


class FakeOperator:
    """The introspection calls of the Python mirror, from a golden fixture."""

    def __init__(self, g, nbr):
        self.N = int(g["N"])
        self._g = g
        self._nbr = nbr

    def pairs(self):
        return self._g["pairs"].astype(np.int32)

    def ranks(self):
        return self._g["rank"].astype(np.int32)

    def leaf_offsets(self):
        return np.concatenate([[0], np.cumsum(self._g["leaf_count"])]).astype(np.int64)

    def neighbors(self, level):
        return self._nbr


@pytest.fixture(scope="module")
def grid16():
    g = gu.load("grid16_q16_tol10")
    nl = 8 ** int(g["levels"])
    return FakeOperator(g, np.full((nl, 26), -1, np.int32))


def test_aca_work_hand_count():
    class Two:
        N = 16

        def pairs(self):
            return np.array([[1, 0, 1], [1, 1, 0]], np.int32)

        def ranks(self):
            return np.array([2, 0], np.int32)

        def leaf_offsets(self):
            return np.array([0, 4, 8, 12, 16, 16, 16, 16, 16], np.int64)

    # pair 0: n = m = 4, rank 2: 3 rows and columns of 8 entries, cross and
    # residual terms 2 * 2 * 1 * 8; pair 1: rank 0, one row and column
    evals, flops = bench.aca_work(Two())
    assert evals == 3 * 8 + 1 * 8
    assert flops == 9 * evals + 2 * 2 * 1 * 8


@pytest.mark.parametrize("engine", sorted(SOURCES))
def test_every_profiled_kernel_has_a_byte_count(grid16, engine):
    src = open(os.path.join(ROOT, "hodlr3d_gb300", "csrc", SOURCES[engine])).read()
    marked = set(re.findall(r'prof->mark\(s, "(\w+)"\)', src))
    lb = bench.level_bytes(grid16, 32, 4, engine)
    assert marked == set(lb), (engine, marked ^ set(lb))
    assert all(v >= 0 for v in lb.values())
    assert bench.engine_of(set(lb)) == engine


def test_factor_bytes_add_up_on_the_golden_tree(grid16):
    H, s, nr = grid16, 4, 32
    g = H._g
    off = H.leaf_offsets()
    d = int(g["levels"])
    ent = 0
    for (j, a, b), r in zip(g["pairs"].tolist(), g["rank"].tolist()):
        w = 8 ** (d - j)
        ent += r * ((off[(a + 1) * w] - off[a * w]) + (off[(b + 1) * w] - off[b * w]))
    assert ent > 0
    N = H.N
    xb, ynl, y = N * nr * s, N * nr * 8, N * nr * 8
    R = g["rank"].astype(np.int64)
    leaf = g["pairs"][:, 0] == d
    t_up, t_leaf = int(R[~leaf].sum()) * nr * s, int(R[leaf].sum()) * nr * s
    gv = bench.level_bytes(H, nr, s, "gemv")
    # A x streams every factor once: V in vt, U in uy (uy also the near blocks)
    fac_vt = gv["vt"] - xb - t_up - t_leaf
    fac_uy = gv["uy"] - t_up - t_leaf - xb - y
    # and so does A^T x: U in ut, V in vy
    fac_ut = gv["ut"] - xb - t_up - t_leaf
    fac_vy = gv["vy"] - t_up - t_leaf - xb - y
    assert fac_vt + fac_ut == ent * s
    assert fac_uy - fac_ut == fac_vy - fac_vt  # the near-field blocks, in both directions
    sm = bench.level_bytes(H, nr, s, "simt")
    parts = sm["tred"] - t_up
    fac_simt = (sm["vtx"] - xb - t_up - parts) + (sm["ut"] - t_up - ynl) + (sm["leaf"] - xb - ynl - y)
    assert fac_simt == ent * s
    tc = bench.level_bytes(H, nr, s, "tc")
    # the tensor cores stream the factors above the leaves and, at the leaf
    # level, the dense blocks of the leaf-level pairs next to the near field
    dense_leaf = 0
    up_ent = 0
    for (j, a, b), r in zip(g["pairs"].tolist(), g["rank"].tolist()):
        w = 8 ** (d - j)
        na, mb = off[(a + 1) * w] - off[a * w], off[(b + 1) * w] - off[b * w]
        if j == d:
            dense_leaf += na * ((mb + 3) // 4 * 4)
        else:
            up_ent += r * (na + mb)
    fac_tc = (tc["ta_slice"] - xb - t_up - parts) + (tc["ut_tc"] - t_up - ynl)
    assert fac_tc == up_ent * s
    assert tc["leaf_rows"] - (fac_uy - fac_ut) - xb - ynl - y == dense_leaf * s
