"""hodlr3d_matvec_noalloc, the matvec for callers that cannot allocate device
memory while they run (a fixed memory budget handed out up front, or an
allocator that must not be re-entered from the computing thread).

It is checked through the C ABI against hodlr3d_matvec on two calls in a row
(the fixed scratch array keeps the first call's contents when the second
runs) and against the reference's own FP64 product of the same operator
(the grid32_q16_tol10 fixture), at the tolerances of the other parity tests;
that a call leaves the device's free memory unchanged (nothing allocated);
and that its size limit is refused cleanly.  Kept in a file that pytest
collects last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(L):
    f = L.hodlr3d_matvec_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                  ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.fixture(scope="module")
def handle():
    from hodlr3d_gb300 import _lib
    from hodlr3d_gb300.workloads import grid_cell_centres
    L = _lib.lib()
    pts = grid_cell_centres(32)  # depth 3: every work buffer of the product is used
    h = ctypes.c_void_p()
    opt = _lib.default_options()
    _lib.check(L.hodlr3d_create(pts.ctypes.data, len(pts), 4, 1.0, 10, 16, ctypes.byref(opt),
                                ctypes.byref(h)))
    _lib.check(L.hodlr3d_assemble(h))
    yield L, h, len(pts)
    L.hodlr3d_destroy(h)


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-6)])
def test_noalloc_matches_matvec_on_two_calls(handle, precision, tol):
    import torch
    from hodlr3d_gb300 import _lib
    L, h, N = handle
    noalloc = _bind(L)
    nrhs = 2
    X = torch.tensor(np.random.default_rng(4).standard_normal((nrhs, N)), device="cuda")
    ref = torch.empty_like(X)
    out = torch.empty_like(X)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(L.hodlr3d_matvec(h, X.data_ptr(), ref.data_ptr(), nrhs, N, precision, stream))
    torch.cuda.synchronize()
    for _ in range(2):
        out.fill_(float("nan"))
        _lib.check(noalloc(h, X.data_ptr(), out.data_ptr(), nrhs, N, precision, stream))
        torch.cuda.synchronize()
        err = (torch.linalg.norm(out - ref, dim=1) / torch.linalg.norm(ref, dim=1)).max().item()
        assert err <= tol, err


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-6)])
def test_noalloc_matches_reference_golden(handle, precision, tol):
    """Against the reference's FP64 product (tests/golden/grid32_q16_tol10),
    on the same charges, two calls in a row."""
    import torch
    from golden_util import load
    from hodlr3d_gb300 import _lib
    from hodlr3d_gb300.workloads import charges_uniform
    L, h, N = handle
    g = load("grid32_q16_tol10")
    assert int(g["N"]) == N
    noalloc = _bind(L)
    x = torch.tensor(charges_uniform(N, seed=1), device="cuda")
    y = torch.empty_like(x)
    ref = torch.tensor(g["matvec"], device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        y.fill_(float("nan"))
        _lib.check(noalloc(h, x.data_ptr(), y.data_ptr(), 1, N, precision, stream))
        torch.cuda.synchronize()
        err = (torch.linalg.norm(y - ref) / torch.linalg.norm(ref)).item()
        assert err <= tol, err


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_allocates_nothing(handle, precision):
    """A call after a warm-up one (which may load the module's code) leaves
    the device's free memory, as cudaMemGetInfo reports it, unchanged."""
    import torch
    from hodlr3d_gb300 import _lib
    L, h, N = handle
    noalloc = _bind(L)
    nrhs = 2  # the most the 64 MiB scratch holds for 32^3 points in the FP64 form
    X = torch.tensor(np.random.default_rng(6).standard_normal((nrhs, N)), device="cuda")
    Y = torch.empty_like(X)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(noalloc(h, X.data_ptr(), Y.data_ptr(), nrhs, N, precision, stream))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        _lib.check(noalloc(h, X.data_ptr(), Y.data_ptr(), nrhs, N, precision, stream))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_refuses_sizes_beyond_its_scratch(handle):
    import torch
    from hodlr3d_gb300 import _lib
    L, h, N = handle
    noalloc = _bind(L)
    nrhs = 64
    X = torch.zeros((nrhs, N), dtype=torch.float64, device="cuda")
    Y = torch.zeros_like(X)
    code = noalloc(h, X.data_ptr(), Y.data_ptr(), nrhs, N, 0, torch.cuda.current_stream().cuda_stream)
    assert code == _lib.ERR_INVALID_ARG
    assert b"scratch" in L.hodlr3d_last_error()
