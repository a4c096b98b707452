"""The matvec inside a CUDA graph: after one eager call on the handle (which
builds the engine's work buffers and tables), hodlr3d_matvec issues only
kernel launches on the caller's stream, so torch.cuda.graph captures it and
every replay recomputes the product of whatever the input buffer then holds.
Each engine is checked: few-column (mixed, 1 and 4 columns, A x and A^T x),
tensor cores (mixed, 32 columns), CUDA cores (FP64)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def op():
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import grid_cell_centres
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(32))
    H.assemble()
    yield H
    H.close()


@pytest.mark.parametrize("precision,nrhs,transpose", [
    ("mixed", 1, False), ("mixed", 4, True), ("mixed", 32, False), ("fp64", 1, False)])
def test_matvec_replays_in_a_cuda_graph(op, precision, nrhs, transpose):
    H = op
    g = torch.Generator(device="cpu").manual_seed(nrhs)
    X = torch.randn(H.N, nrhs, generator=g, dtype=torch.float64).cuda()
    X2 = torch.randn(H.N, nrhs, generator=g, dtype=torch.float64).cuda()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        H.matvec(X, precision, transpose=transpose)  # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        Y = H.matvec(X, precision, transpose=transpose)
    X.copy_(X2)
    graph.replay()
    torch.cuda.synchronize()
    H.device_status()
    assert torch.equal(Y, H.matvec(X2, precision, transpose=transpose))
