"""Ragged and empty inputs: a clustered point set leaves most leaves empty and
the others with arbitrary populations.  Every engine and precision must still
agree with the FP64 form (which the golden tests pin to the reference): the
few-column, tensor-core (refused: leaves not multiples of 4) and CUDA-core
engines, A x and A^T x, 1..64 columns, and fp64x."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clustered():
    from hodlr3d_gb300 import HODLR3D
    rng = np.random.default_rng(5)
    # a slab z < -0.5: 16 of the 64 leaves hold the points, 48 are empty
    pts = np.column_stack([rng.uniform(-1.0, 1.0, 1500), rng.uniform(-1.0, 1.0, 1500),
                           rng.uniform(-1.0, -0.5, 1500)])
    H = HODLR3D(4, 1.0, 10, 16, pts)
    H.assemble()
    yield H
    H.close()


def colerr(a, b):
    return (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()


def test_tree_has_empty_and_ragged_leaves(clustered):
    cnt = np.diff(clustered.leaf_offsets())
    assert (cnt == 0).sum() >= len(cnt) // 2 and (cnt % 4 != 0).any() and cnt.max() <= 200


@pytest.mark.parametrize("transpose", [False, True])
@pytest.mark.parametrize("nrhs", [1, 3, 8, 64])
def test_engines_agree_on_ragged_trees(clustered, nrhs, transpose):
    H = clustered
    X = torch.tensor(np.random.default_rng(nrhs).standard_normal((H.N, nrhs)), device="cuda")
    y64 = H.matvec(X, "fp64", transpose=transpose)
    for eng in ("auto", "simt", "gemv"):
        H.set_engine(eng)
        y = H.matvec(X, "mixed", transpose=transpose)
        assert colerr(y, y64) <= 2e-6, eng
    H.set_engine("tc")
    if not transpose:
        with pytest.raises(RuntimeError, match="tensor-core engine"):
            H.matvec(X, "mixed")
    H.set_engine("auto")
    yx = H.matvec(X, "fp64x", transpose=transpose)
    H.device_status()
    assert colerr(yx, y64) <= 1e-12


def test_dense_rows_outside_the_point_set(clustered):
    """Row ids outside [0, n): the Python mirror refuses them; through the C ABI
    (device ids, checked by the kernel) their outputs are NaN and the others
    are unaffected."""
    from hodlr3d_gb300 import _lib
    H = clustered
    x = torch.tensor(np.random.default_rng(2).standard_normal(H.N), device="cuda")
    with pytest.raises(ValueError):
        H.dense_rows([0, H.N], x)
    rows = torch.tensor([3, -1, H.N, 7], dtype=torch.int64, device="cuda")
    y = torch.empty(4, dtype=torch.float64, device="cuda")
    st = _lib.lib().hodlr3d_dense_rows(H.handle, rows.data_ptr(), 4, x.data_ptr(), y.data_ptr(),
                                       1, H.N, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.OK
    torch.cuda.synchronize()
    H.device_status()
    good = H.dense_rows([3, 7], x)
    assert torch.isnan(y[1]) and torch.isnan(y[2])
    assert torch.equal(y[[0, 3]], good)
