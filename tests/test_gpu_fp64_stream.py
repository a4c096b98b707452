"""The FP64 form streamed from FP64 factors grouped by box
(hodlr3d_gb300/csrc/matvec_f64.cu), the automatic engine of the FP64
product: against the CUDA-core FP64 kernels (the same operator, another
summation order: 1e-14), against the reference's own FP64 product (1e-12 for
the algebraic kernels), forward and transposed, several columns (one pass
each)."""
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


def _engine_kernels(H, fn):
    H.set_profiling(True)
    fn()
    torch.cuda.synchronize()
    rep = H.profile_report()
    H.set_profiling(False)
    return set(rep)


@pytest.mark.parametrize("transpose", [False, True])
def test_fp64_stream_matches_cuda_core_fp64(case, transpose):
    g, H = case
    X = torch.tensor(np.random.default_rng(5).standard_normal((H.N, 3)), device="cuda")
    names = _engine_kernels(H, lambda: H.matvec(X, "fp64", transpose=transpose))
    assert ("vy64" if transpose else "uy64") in names, names
    ys = H.matvec(X, "fp64", transpose=transpose)
    H.set_engine("simt")
    yc = H.matvec(X, "fp64", transpose=transpose)
    H.set_engine("auto")
    err = (torch.linalg.norm(ys - yc, dim=0) / torch.linalg.norm(yc, dim=0)).max().item()
    assert err <= 1e-14, err
    # one column at a time gives the same columns (one pass per column)
    y1 = H.matvec(X[:, 1].contiguous(), "fp64", transpose=transpose)
    assert torch.equal(y1, ys[:, 1])


def test_fp64_stream_matches_reference(case):
    from hodlr3d_gb300.workloads import charges_uniform
    g, H = case
    q = charges_uniform(H.N, seed=1)
    y = H.MatVecProduct(q, precision="fp64")
    err = np.linalg.norm(y - g["matvec"]) / np.linalg.norm(g["matvec"])
    assert err <= (1e-12 if int(g["kernel"]) in ALGEBRAIC else 1e-10), err
