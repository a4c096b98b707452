"""Configuration C4 at its full size: 64^3 grid, 1/r (Qchoice 16), tol 1e-10;
mixed iterative-refinement GMRES for 32 right-hand sides against a known
solution, and the adjoint solve (its residual through the transpose
product)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c4():
    from hodlr3d_gb300 import HODLR3D
    from hodlr3d_gb300.workloads import grid_cell_centres
    H = HODLR3D(4, 1.0, 10, 16, grid_cell_centres(64))
    H.assemble()
    yield H
    H.close()


def test_c4_mixed_gmres_known_solution(c4):
    from hodlr3d_gb300.workloads import charges_uniform
    H = c4
    xt = torch.tensor(charges_uniform(H.N, nrhs=32, seed=3), device="cuda")
    b = H.matvec(xt, "fp64")
    x, info = H.gmres(b, tol=1e-10, restart=30, precision="mixed")
    assert info["converged"], info
    r = H.matvec(x, "fp64") - b
    assert (torch.linalg.norm(r, dim=0) / torch.linalg.norm(b, dim=0)).max().item() <= 1e-9
    err = (torch.linalg.norm(x - xt, dim=0) / torch.linalg.norm(xt, dim=0)).max().item()
    assert err <= 1e-8, err


def test_c4_adjoint_solve(c4):
    from hodlr3d_gb300.workloads import charges_normal
    H = c4
    g = torch.tensor(charges_normal(H.N, nrhs=2, seed=4), device="cuda")
    lam, info = H.gmres(g, tol=1e-10, restart=30, transpose=True)
    assert info["converged"], info
    r = H.matvec(lam, "fp64", transpose=True) - g
    assert (torch.linalg.norm(r, dim=0) / torch.linalg.norm(g, dim=0)).max().item() <= 1e-9


def test_c4_gradient_of_half_norm_squared(c4):
    """L = 0.5 |x|^2 with x = solve(b), b = A x_true, x_true U[0,1): the
    gradient dL/db that autograd returns (the adjoint solve A^T lam = x,
    hodlr3d_gb300/autograd.py) is checked two ways.

    1. Central finite differences, h = 1e-6, on 16 random components:
       (L(b + h e_i) - L(b - h e_i)) / (2 h).  Each L(b +- h e_i) is a GMRES
       solve warm-started at the base solution x0 (the correction d solves
       A d = (b +- h e_i) - A x0, to 1e-10 of its own right-hand side), and
       the difference of the two values of L is formed without cancellation,
       0.5 (d+ - d-) . (2 x0 + d+ + d-): L itself is ~4e4, so differencing two
       rounded values of L would lose the 1e-6 it is compared at.
       Agreement: within 1e-6 of max |dL/db|.
    2. The dense FP64 adjoint on 4096 sampled rows: K is symmetric, so
       (K^T lam)[rows] is the dense FP64 product of those rows of K with lam,
       which must reproduce x0[rows] (to the ACA tolerance).
    """
    from hodlr3d_gb300 import autograd
    from hodlr3d_gb300.workloads import charges_uniform
    H = c4
    N = H.N
    xt = torch.tensor(charges_uniform(N, seed=5), device="cuda")
    b = H.matvec(xt, "fp64")
    opts = dict(tol=1e-10, restart=30, precision="mixed")
    bb = b.clone().requires_grad_(True)
    x = autograd.solve(H, bb, **opts)
    L = 0.5 * (x * x).sum()
    L.backward()
    grad = bb.grad.detach()
    x0 = x.detach()

    h = 1e-6
    idx = np.random.default_rng(17).choice(N, 16, replace=False)
    r0 = b - H.matvec(x0, "fp64")
    R = r0[:, None].repeat(1, 32)
    for k, i in enumerate(idx):
        R[i, 2 * k] += h
        R[i, 2 * k + 1] -= h
    D, info = H.gmres(R, **opts)
    assert info["converged"], info
    dp, dm = D[:, 0::2], D[:, 1::2]
    fd = 0.5 * ((dp - dm) * (2 * x0[:, None] + dp + dm)).sum(dim=0) / (2 * h)
    g = grad[torch.as_tensor(idx, device="cuda")]
    scale = grad.abs().max().item()
    dev = (fd - g).abs().max().item()
    assert dev <= 1e-6 * scale, (dev, scale)

    rows = np.sort(np.random.default_rng(18).choice(N, 4096, replace=False))
    kt_lam = H.dense_rows(rows, grad)
    ref = x0[torch.as_tensor(rows, device="cuda")]
    err = (torch.linalg.norm(kt_lam - ref) / torch.linalg.norm(ref)).item()
    assert err <= 1e-8, err
