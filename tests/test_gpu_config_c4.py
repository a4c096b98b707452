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
