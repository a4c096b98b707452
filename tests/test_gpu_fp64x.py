"""The FP64-accurate form in FP32-pair arithmetic (HODLR3D_FP64X): every FP64
factor and near-field entry as hi + lo FP32 values, exact FP32 products and
compensated sums.  It must agree with the FP64 form (and so with the
reference's FP64 products) to FP64-level accuracy: 1e-12 relative here, ~1e-14
expected; every golden case, A x and A^T x, 1..7 columns."""
import numpy as np
import pytest
import torch

from golden_util import golden_names, load, points_of

pytestmark = pytest.mark.gpu

ALGEBRAIC = {2, 3, 4, 6, 7, 8, 16}


@pytest.fixture(scope="module", params=golden_names())
def case(request):
    from hodlr3d_gb300 import HODLR3D
    g = load(request.param)
    H = HODLR3D(int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), points_of(g),
                diag_override=float(g["diag"]))
    H.assemble()
    yield g, H
    H.close()


def colerr(a, b):
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("nrhs", [1, 2, 4, 7])
def test_fp64x_matches_fp64(case, nrhs, transpose):
    g, H = case
    X = torch.tensor(np.random.default_rng(nrhs).standard_normal((H.N, nrhs)), device="cuda")
    y64 = H.matvec(X, "fp64", transpose=transpose)
    yx = H.matvec(X, "fp64x", transpose=transpose)
    H.device_status()
    assert colerr(yx, y64) <= 1e-12
    # columns are independent of the batch they travel in
    y1 = H.matvec(X[:, -1:].contiguous(), "fp64x", transpose=transpose)
    assert torch.equal(y1[:, 0], yx[:, -1])


def test_fp64x_matches_reference_fp64(case):
    from hodlr3d_gb300.workloads import charges_uniform
    g, H = case
    q = charges_uniform(H.N, seed=1)
    y = H.MatVecProduct(q, precision="fp64x")
    ref = g["matvec"]
    tol = 1e-12 if int(g["kernel"]) in ALGEBRAIC else 1e-10
    assert np.linalg.norm(y - ref) <= tol * np.linalg.norm(ref)


def test_fp64x_gmres_matches_fp64(case):
    """Plain GMRES on fp64x products converges where it does on FP64 products,
    in as many iterations give or take one, to a solution whose FP64 residual
    meets the tolerance."""
    g, H = case
    b = torch.tensor(np.random.default_rng(5).random(H.N), device="cuda")
    tol = 1e-10
    x64, i64 = H.gmres(b, maxit=300, tol=tol, restart=30, precision="fp64", raise_on_failure=False)
    if not i64["converged"]:
        pytest.skip("GMRES(30) does not reach the tolerance on this operator")
    xx, ix = H.gmres(b, maxit=300, tol=tol, restart=30, precision="fp64x", raise_on_failure=False)
    assert ix["converged"]
    assert abs(ix["iterations"] - i64["iterations"]) <= 1
    res = (torch.linalg.norm(b - H.matvec(xx, "fp64")) / torch.linalg.norm(b)).item()
    assert res <= 2 * tol, res


def test_fp64x_without_fp32_copies_is_the_fp64_form(tmp_path):
    """keep_fp32 = 0: no FP32 copies to pair with, so fp64x products are the
    FP64 form's, bit for bit; a factor file saved from such a handle loads
    into one with the copies (the file holds the FP64 factors)."""
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import grid_cell_centres
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(16), keep_fp32=False)
    H.assemble()
    X = torch.tensor(np.random.default_rng(9).standard_normal((H.N, 3)), device="cuda")
    y64 = H.matvec(X, "fp64")
    assert torch.equal(H.matvec(X, "fp64x"), y64)
    with pytest.raises(RuntimeError, match="keep_fp32"):
        H.matvec(X, "mixed")
    path = tmp_path / "op.h3d"
    H.save(path)
    G = HODLR3D.load(path)
    try:
        # G keeps the FP32 copies: its FP64 form streams FP64 factors grouped
        # like them (another summation order than the CUDA-core kernels)
        assert colerr(G.matvec(X, "fp64"), y64) <= 1e-14
        assert colerr(G.matvec(X, "fp64x"), y64) <= 1e-12
    finally:
        G.close()
        H.close()


def test_fp64x_under_forced_engines(case):
    """Forcing the CUDA-core engine gives the FP64 form; the tensor cores have
    no FP64-accurate form and refuse it."""
    g, H = case
    X = torch.tensor(np.random.default_rng(2).standard_normal((H.N, 2)), device="cuda")
    H.set_engine("simt")
    ys = H.matvec(X, "fp64x")
    y64 = H.matvec(X, "fp64")  # the CUDA-core FP64 form
    H.set_engine("tc")
    with pytest.raises(RuntimeError, match="FP64-accurate"):
        H.matvec(X, "fp64x")
    H.set_engine("auto")
    assert torch.equal(ys, y64)
