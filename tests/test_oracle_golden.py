"""Pins the CPU oracle against the reference's own outputs (tests/golden/).

The fixtures were produced by the HODLR3D reference sources themselves
(tests/golden/make_golden.py).  Integer results (leaf order, neighbour slots,
interaction-list sets, ACA ranks and pivots) must be identical; the matvec
agrees to rounding (1e-13 relative) and the GMRES history to 1e-6 relative.
"""
import numpy as np
import pytest

from golden_util import golden_names, load, pair_keys, pivot_crc_per_box, points_of
from oracle.oracle import Oracle

NAMES = golden_names()


@pytest.fixture(scope="module", params=NAMES)
def case(request):
    g = load(request.param)
    pts = points_of(g)
    o = Oracle(pts, int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), float(g["diag"]))
    o.assemble()
    return g, o


def test_fixture_set_complete():
    assert len(NAMES) >= 7


def test_depth_and_kii(case):
    g, o = case
    assert o.levels == int(g["levels"])
    if int(g["kernel"]) == 16:
        assert abs(o.kii - g["kii"][0]) <= 2e-16 * abs(g["kii"][0])


def test_leaf_order_bit_exact(case):
    g, o = case
    assert np.array_equal(o.perm(), g["perm"])
    off = o.box_offsets(o.levels)
    assert np.array_equal(np.diff(off), g["leaf_count"])


def test_neighbour_slots_bit_exact(case):
    g, o = case
    ref = g["nbr"].astype(np.int32).reshape(-1, 26)
    start = 0
    for j in range(o.levels + 1):
        nb = 8 ** j
        assert np.array_equal(o.neighbors(j), ref[start:start + nb]), f"level {j}"
        start += nb


def test_interaction_lists_bit_exact(case):
    g, o = case
    P = o.pairs()
    assert np.array_equal(np.bincount(P[:, 0], minlength=o.levels + 1), g["pair_count_per_level"])
    import hashlib
    assert hashlib.sha256(P.astype(np.int32).tobytes()).hexdigest() == str(g["pairs_sha256"])
    if "pairs" in g:
        assert np.array_equal(pair_keys(P), pair_keys(g["pairs"].astype(np.int32)))


def test_aca_ranks_and_pivots_identical(case):
    g, o = case
    ranks = o.ranks()
    assert np.array_equal(ranks, g["rank"].astype(np.int32))
    rows, cols = o.pivots()
    if "row_piv" in g:
        assert np.array_equal(rows, g["row_piv"].astype(np.int32))
        assert np.array_equal(cols, g["col_piv"].astype(np.int32))
    else:
        crc = pivot_crc_per_box(o.pairs(), ranks, rows, cols)
        assert np.array_equal(crc, g["piv_crc_box"])


def test_matvec_matches_reference(case):
    from hodlr3d_gb300.workloads import charges_uniform
    g, o = case
    q = charges_uniform(o.N, seed=1)
    y = o.matvec(q)
    ref = g["matvec"]
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)
    y_uv = o.matvec_uv(q)
    assert np.linalg.norm(y_uv - ref) <= 1e-12 * np.linalg.norm(ref)


def test_memory_and_max_rank(case):
    g, o = case
    mem, maxrank = g["stats"]
    assert o.memory_entries() == mem
    assert o.max_rank() == int(maxrank)


def test_gmres_history(case):
    g, o = case
    if "gmres_hist" not in g:
        pytest.skip("no GMRES run for this case")
    from hodlr3d_gb300.workloads import charges_uniform
    q = charges_uniform(o.N, seed=1)
    x, hist, nit = o.gmres(q, maxit=int(g["gmres_maxit"]), tol=1e-10)
    assert nit == int(g["gmres_nit"][0])
    assert np.allclose(hist, g["gmres_hist"], rtol=1e-6, atol=1e-15)
    # The reference solves the small rotated Hessenberg system by pivoted QR and
    # the oracle by back substitution; on a run that stops at maxit without
    # converging that system is ill-conditioned, so x agrees less tightly.
    converged = g["gmres_hist"][-1] <= 1e-10
    tol = 1e-9 if converged else 1e-6
    assert np.linalg.norm(x - g["gmres_x"]) <= tol * np.linalg.norm(g["gmres_x"])
