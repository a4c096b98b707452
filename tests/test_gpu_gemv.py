"""The few-column engine (1..4 right-hand sides, FP32 factors streamed once,
FP32 FMAs, FP64 across segments) of the mixed-precision matvec: A x and A^T x
against the CUDA-core engine, the reference's FP64 matvec and the oracle's
transpose, on every golden case (grid and random points, whose leaf
populations are not multiples of 4)."""
import numpy as np
import pytest
import torch

from golden_util import golden_names, load, points_of

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=golden_names())
def case(request):
    from hodlr3d_gb300 import HODLR3D
    g = load(request.param)
    pts = points_of(g)
    H = HODLR3D(int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), pts,
                diag_override=float(g["diag"]))
    H.assemble()
    yield g, H, pts
    H.close()


def colerr(a, b):
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("nrhs", [1, 2, 3, 4, 7])
def test_gemv_matches_simt_engine(case, nrhs, transpose):
    g, H, _ = case
    X = torch.tensor(np.random.default_rng(nrhs).standard_normal((H.N, nrhs)), device="cuda")
    H.set_engine("simt")
    ys = H.matvec(X, "mixed", transpose=transpose)
    H.set_engine("gemv")
    yg = H.matvec(X, "mixed", transpose=transpose)
    H.set_engine("auto")
    ya = H.matvec(X, "mixed", transpose=transpose)
    H.device_status()
    assert colerr(yg, ys) <= 2e-6
    tc_tree = bool((np.diff(H.leaf_offsets()) % 4 == 0).all()) and int(np.diff(H.leaf_offsets()).max()) <= 128
    if transpose or nrhs <= 4 or not tc_tree:
        # the automatic choice: A^T x up to 32 columns, A x up to 4 (up to 32
        # on trees the tensor-core engine does not take)
        assert torch.equal(ya, yg)
    # columns are independent: the product of one column alone is the same
    H.set_engine("gemv")
    y1 = H.matvec(X[:, :1].contiguous(), "mixed", transpose=transpose)
    H.set_engine("auto")
    assert torch.equal(y1[:, 0], yg[:, 0])


def test_gemv_matches_reference_fp64(case):
    from hodlr3d_gb300.workloads import charges_uniform
    g, H, _ = case
    q = charges_uniform(H.N, seed=1)
    H.set_engine("gemv")
    y = H.MatVecProduct(q, precision="mixed")
    H.set_engine("auto")
    ref = g["matvec"]
    assert np.linalg.norm(y - ref) <= 2e-6 * np.linalg.norm(ref)


def test_gemv_transpose_matches_oracle(case):
    from oracle.oracle import Oracle
    g, H, pts = case
    o = Oracle(pts, int(g["nP1D"]), float(g["L"]), int(g["tol_pow"]), int(g["kernel"]), float(g["diag"]))
    o.assemble()
    x = np.random.default_rng(7).standard_normal(H.N)
    H.set_engine("gemv")
    yt = H.matvec_transpose(torch.tensor(x, device="cuda"), precision="mixed").cpu().numpy()
    H.set_engine("auto")
    ref = o.matvec_uv_t(x)
    assert np.linalg.norm(yt - ref) <= 2e-6 * np.linalg.norm(ref)


def test_gemv_adjoint_identity(case):
    """<A x, z> = <x, A^T z> for the mixed forms, to the FP32 rounding of the
    two products (scaled by |A x| |z|)."""
    g, H, _ = case
    rng = np.random.default_rng(11)
    x = torch.tensor(rng.standard_normal((H.N, 2)), device="cuda")
    z = torch.tensor(rng.standard_normal((H.N, 2)), device="cuda")
    H.set_engine("gemv")
    ax = H.matvec(x, "mixed")
    atz = H.matvec(z, "mixed", transpose=True)
    H.set_engine("auto")
    lhs = (ax * z).sum(dim=0)
    rhs = (x * atz).sum(dim=0)
    scale = torch.linalg.norm(ax, dim=0) * torch.linalg.norm(z, dim=0)
    assert ((lhs - rhs).abs() <= 2e-6 * scale).all(), (lhs, rhs, scale)


def test_gemv_takes_fp64_as_the_fp64_stream(case):
    """Forced few-column engine with the FP64 form: the FP64 streaming kernels
    (FP64 factors grouped by box), the same product as the automatic choice."""
    g, H, _ = case
    x = torch.ones(H.N, 1, dtype=torch.float64, device="cuda")
    ya = H.matvec(x, "fp64")
    H.set_engine("gemv")
    yg = H.matvec(x, "fp64")
    H.set_engine("auto")
    assert torch.equal(ya, yg)
