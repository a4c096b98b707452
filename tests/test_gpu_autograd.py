"""torch.autograd through the matvec and the solve (hodlr3d_gb300/autograd.py).

The products are linear, so their gradients are exact adjoints: the backward
of y = A x is A^T g (the transpose product), the backward of x = A^-1 b is the
adjoint solve A^-T g.  Checked through the adjoint identities
<grad, v> = <g, A v> and <grad, c> = <g, A^-1 c> for random directions, and,
for the symmetric 1/r kernel, against the dense FP64 product K g of sampled
rows (K is symmetric, so K^T g = K g up to the compression tolerance)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def op():
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import grid_cell_centres
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(16))
    H.assemble()
    yield H
    H.close()


def rand(H, nrhs, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(H.N, nrhs, generator=g, dtype=torch.float64).cuda()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-6)])
def test_matvec_backward_is_the_transpose(op, precision, tol):
    from hodlr3d_gb300 import autograd
    H = op
    x = rand(H, 3, 1).requires_grad_(True)
    w = rand(H, 3, 2)
    loss = (autograd.matvec(H, x, precision) * w).sum()
    loss.backward()
    v = rand(H, 3, 3)
    av = H.matvec(v, precision)
    lhs = (x.grad * v).sum(dim=0)                      # <A^T w, v>
    rhs = (w * av).sum(dim=0)                          # <w, A v>
    # inner products of random vectors cancel: the bound scales with |w| |A v|
    scale = torch.linalg.norm(w, dim=0) * torch.linalg.norm(av, dim=0)
    assert ((lhs - rhs).abs() <= tol * scale).all(), (lhs, rhs, scale)
    # the transpose product itself
    assert torch.equal(x.grad, H.matvec(w, precision, transpose=True))


def test_matvec_gradient_matches_dense_rows(op):
    from hodlr3d_gb300 import autograd
    H = op
    x = rand(H, 1, 4)[:, 0].requires_grad_(True)
    w = rand(H, 1, 5)[:, 0]
    (autograd.matvec(H, x, "fp64") * w).sum().backward()
    rows = np.sort(np.random.default_rng(6).choice(H.N, 256, replace=False))
    dense = H.dense_rows(rows, w)                      # (K w)[rows] = (K^T w)[rows]
    got = x.grad[torch.as_tensor(rows, device="cuda")]
    err = (torch.linalg.norm(got - dense) / torch.linalg.norm(dense)).item()
    assert err <= 1e-8, err


@pytest.mark.parametrize("precision,stol,tol", [("fp64", 1e-12, 1e-8), ("mixed", 1e-10, 1e-8)])
def test_solve_backward_is_the_adjoint_solve(op, precision, stol, tol):
    from hodlr3d_gb300 import autograd
    H = op
    b = rand(H, 2, 7).requires_grad_(True)
    w = rand(H, 2, 8)
    x = autograd.solve(H, b, tol=stol, precision=precision)
    (x * w).sum().backward()
    c = rand(H, 2, 9)
    xc, info = H.gmres(c, tol=stol, restart=30, precision=precision)
    assert info["converged"]
    lhs = (b.grad * c).sum(dim=0)                      # <A^-T w, c>
    rhs = (w * xc).sum(dim=0)                          # <w, A^-1 c>
    scale = torch.linalg.norm(w, dim=0) * torch.linalg.norm(xc, dim=0)
    assert ((lhs - rhs).abs() <= tol * scale).all(), (lhs, rhs, scale)
    # the gradient solves A^T lambda = w
    res = H.matvec(b.grad, "fp64", transpose=True) - w
    rel = (torch.linalg.norm(res, dim=0) / torch.linalg.norm(w, dim=0)).max().item()
    assert rel <= 10 * stol, rel


def test_transposed_solve_backward_solves_with_a(op):
    """solve(..., transpose=True) gives x = A^-T b; its gradient solves A lambda = w."""
    from hodlr3d_gb300 import autograd
    H = op
    b = rand(H, 1, 13).requires_grad_(True)
    w = rand(H, 1, 14)
    x = autograd.solve(H, b, tol=1e-12, transpose=True)
    res = H.matvec(x.detach(), "fp64", transpose=True) - b.detach()
    assert torch.linalg.norm(res) <= 1e-10 * torch.linalg.norm(b.detach())
    (x * w).sum().backward()
    res = H.matvec(b.grad, "fp64") - w
    assert torch.linalg.norm(res) <= 1e-10 * torch.linalg.norm(w)


def test_solve_central_difference(op):
    """d/de <w, A^-1 (b + e c)> at e = 0 by central differences (exact for a
    linear map up to the solver tolerance) against <grad_b, c>."""
    from hodlr3d_gb300 import autograd
    H = op
    b = rand(H, 1, 10)[:, 0].requires_grad_(True)
    w = rand(H, 1, 11)[:, 0]
    c = rand(H, 1, 12)[:, 0]
    (autograd.solve(H, b, tol=1e-13) * w).sum().backward()
    e = 1e-3
    xp, _ = H.gmres(b.detach() + e * c, tol=1e-13, restart=30)
    xm, _ = H.gmres(b.detach() - e * c, tol=1e-13, restart=30)
    fd = ((w * xp).sum() - (w * xm).sum()) / (2 * e)
    an = (b.grad * c).sum()
    scale = (torch.linalg.norm(w) * torch.linalg.norm(b.grad) * torch.linalg.norm(c)
             / torch.linalg.norm(b.grad)).item()
    assert abs(fd.item() - an.item()) <= 1e-7 * scale, (fd.item(), an.item(), scale)
