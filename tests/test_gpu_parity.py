"""CUDA path against the reference's golden outputs and the CPU oracle.

Integer results (leaf order, neighbour slots, interaction lists, ACA ranks
and pivots) must be identical for the algebraic kernels; for kernels built on
exp/log/cos the device math library may differ from the host's in the last
bit, so ranks may differ on a few borderline blocks (bounded below).  The
FP64 matvec matches the reference's to 1e-12 relative; the mixed form is
within 2e-6 of it.
"""
import numpy as np
import pytest

from golden_util import golden_names, load, pair_keys, pivot_crc_per_box, points_of

pytestmark = pytest.mark.gpu

ALGEBRAIC = {2, 3, 4, 6, 7, 8, 16}


@pytest.fixture(scope="module", params=golden_names())
def gcase(request):
    from hodlr3d_gb300 import HODLR3D
    g = load(request.param)
    pts = points_of(g)
    H = HODLR3D(int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), pts,
                diag_override=float(g["diag"]))
    H.assemble()
    yield g, H, pts
    H.close()


def test_tree_leaf_order_bit_exact(gcase):
    g, H, _ = gcase
    assert H.levels == int(g["levels"])
    assert np.array_equal(H.perm(), g["perm"])
    assert np.array_equal(np.diff(H.leaf_offsets()), g["leaf_count"])


def test_neighbour_slots_bit_exact(gcase):
    g, H, _ = gcase
    ref = g["nbr"].astype(np.int32).reshape(-1, 26)
    start = 0
    for j in range(H.levels + 1):
        nb = 8 ** j
        assert np.array_equal(H.neighbors(j), ref[start:start + nb]), f"level {j}"
        start += nb


def test_interaction_lists_bit_exact(gcase):
    import hashlib
    g, H, _ = gcase
    P = H.pairs()
    assert np.array_equal(np.bincount(P[:, 0], minlength=H.levels + 1), g["pair_count_per_level"])
    assert hashlib.sha256(P.astype(np.int32).tobytes()).hexdigest() == str(g["pairs_sha256"])


def test_aca_ranks_and_pivots(gcase):
    g, H, _ = gcase
    ranks = H.ranks()
    ref = g["rank"].astype(np.int32)
    if int(g["kernel"]) in ALGEBRAIC:
        assert np.array_equal(ranks, ref)
        rows, cols = H.pivots()
        if "row_piv" in g:
            assert np.array_equal(rows, g["row_piv"].astype(np.int32))
            assert np.array_equal(cols, g["col_piv"].astype(np.int32))
        else:
            assert np.array_equal(pivot_crc_per_box(H.pairs(), ranks, rows, cols), g["piv_crc_box"])
    else:
        diff = np.abs(ranks - ref)
        assert (diff > 0).mean() <= 0.02 and diff.max() <= 3


def test_matvec_fp64_matches_reference(gcase):
    from hodlr3d_gb300.workloads import charges_uniform
    g, H, _ = gcase
    q = charges_uniform(H.N, seed=1)
    y = H.MatVecProduct(q, precision="fp64")
    ref = g["matvec"]
    err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
    tol = 1e-12 if int(g["kernel"]) in ALGEBRAIC else 1e-10
    assert err <= tol, err


def test_matvec_mixed_accuracy(gcase):
    from hodlr3d_gb300.workloads import charges_uniform
    g, H, _ = gcase
    q = charges_uniform(H.N, seed=1)
    y = H.MatVecProduct(q, precision="mixed")
    ref = g["matvec"]
    err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
    assert err <= 2e-6, err


def test_multi_rhs_columns_match_single(gcase):
    from hodlr3d_gb300.workloads import charges_normal
    g, H, _ = gcase
    Q = charges_normal(H.N, nrhs=5, seed=3)
    Y = H.MatVecProduct(Q, precision="fp64")
    for c in range(5):
        y1 = H.MatVecProduct(Q[:, c], precision="fp64")
        assert np.linalg.norm(Y[:, c] - y1) <= 1e-14 * np.linalg.norm(y1)


def test_host_layouts_agree(gcase):
    """Rows (C order, hodlr3d_matvec_host_rows) and columns (Fortran order,
    hodlr3d_matvec_host) of the same right-hand sides give the same product,
    with and without a caller-provided output array."""
    from hodlr3d_gb300.workloads import charges_normal
    g, H, _ = gcase
    for prec in ("fp64", "mixed"):
        Q = np.ascontiguousarray(charges_normal(H.N, nrhs=20, seed=4))
        Yc = H.MatVecProduct(Q, precision=prec)
        Yf = H.MatVecProduct(np.asfortranarray(Q), precision=prec)
        out = np.empty_like(Q)
        Yo = H.MatVecProduct(Q, precision=prec, out=out)
        assert Yo is out
        assert np.array_equal(Yc, Yf) and np.array_equal(Yc, out)


def test_transpose_matches_oracle(gcase):
    import torch
    from oracle.oracle import Oracle
    g, H, pts = gcase
    o = Oracle(pts, int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), float(g["diag"]))
    o.assemble()
    x = np.random.default_rng(7).standard_normal(H.N)
    yt = H.matvec_transpose(torch.tensor(x, device="cuda")).cpu().numpy()
    ref = o.matvec_uv_t(x)
    # transcendental kernels: a borderline block may take other pivots on the
    # device, so the two operators agree to the ACA tolerance, not to rounding
    tol = 1e-12 if int(g["kernel"]) in ALGEBRAIC else 10.0 ** (2 - int(g["tol_pow"]))
    assert np.linalg.norm(yt - ref) <= tol * np.linalg.norm(ref)
    # <A x, z> == <x, A^T z>
    z = np.random.default_rng(8).standard_normal(H.N)
    ax = H.MatVecProduct(x)
    atz = H.matvec_transpose(torch.tensor(z, device="cuda")).cpu().numpy()
    assert abs(ax @ z - x @ atz) <= 1e-12 * np.linalg.norm(ax) * np.linalg.norm(z)


def test_dense_rows_against_oracle(gcase):
    import torch
    from oracle.oracle import Oracle
    g, H, pts = gcase
    o = Oracle(pts, int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), float(g["diag"]))
    rows = np.random.default_rng(1).choice(H.N, 64, replace=False)
    x = np.random.default_rng(2).random(H.N)
    yd = H.dense_rows(rows, torch.tensor(x, device="cuda")).cpu().numpy()
    yo = o.dense_rows(rows, x)
    assert np.linalg.norm(yd - yo) <= 1e-13 * np.linalg.norm(yo)


def test_gmres_history_matches_reference(gcase):
    from hodlr3d_gb300 import classGMRES
    from hodlr3d_gb300.workloads import charges_uniform
    g, H, _ = gcase
    if "gmres_hist" not in g:
        pytest.skip("no GMRES run for this case")
    q = charges_uniform(H.N, seed=1)
    x, err, nit, e = classGMRES().gmres(H, q, int(g["gmres_maxit"]), 1e-10)
    ref = g["gmres_hist"]
    assert nit == int(g["gmres_nit"][0])
    n = min(len(e), len(ref))
    # a run that stagnates on an ill-conditioned transcendental kernel amplifies
    # the last-bit differences of the device exp into the later residuals
    rtol = 1e-6 if int(g["kernel"]) in ALGEBRAIC else 1e-2
    assert np.allclose(np.array(e[:n]), ref[:n], rtol=rtol, atol=1e-14)
    if ref[-1] <= 1e-10:
        assert np.linalg.norm(x - g["gmres_x"]) <= 1e-9 * np.linalg.norm(g["gmres_x"])


def test_aca_capacity_retries_and_small_workspace_keep_ranks():
    """A rank capacity of 8 and a 64 MiB workspace: most pairs above the
    leaves reach the capacity and run again (capacities 8 -> 16 -> ... up to
    their rank), the assembly takes many batches, and ranks, pivots and the
    FP64 product are those of the reference all the same (grid32_q16_tol10)."""
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import charges_uniform
    g = load("grid32_q16_tol10")
    H = HODLR3D(int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), points_of(g),
                diag_override=float(g["diag"]), aca_workspace_bytes=64 << 20, rank_cap=8)
    try:
        H.assemble()
        st = H.stats()
        assert st["aca_batches"] > 4, st["aca_batches"]
        ranks = H.ranks()
        assert np.array_equal(ranks, g["rank"].astype(np.int32))
        rows, cols = H.pivots()
        if "row_piv" in g:
            assert np.array_equal(rows, g["row_piv"].astype(np.int32))
            assert np.array_equal(cols, g["col_piv"].astype(np.int32))
        else:
            assert np.array_equal(pivot_crc_per_box(H.pairs(), ranks, rows, cols), g["piv_crc_box"])
        q = charges_uniform(H.N, seed=1)
        y = H.MatVecProduct(q, precision="fp64")
        assert np.linalg.norm(y - g["matvec"]) <= 1e-12 * np.linalg.norm(g["matvec"])
    finally:
        H.close()
