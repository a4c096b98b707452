"""torch.autograd wrappers of the matvec and the solve.

* ``matvec(H, x)``: y = A x; its backward is the hand-written transpose
  product A^T g (V (U^T g) on the compressed pairs, transposed near field).
* ``solve(H, b)``: x = A^{-1} b by GMRES; its backward is the adjoint solve
  A^T lambda = g, and grad_b = lambda (``transpose=True`` solves A^T x = b,
  whose backward solves with A).

Both take CUDA float64 tensors of shape (N,) or (N, nrhs).  A forward or
adjoint solve that does not reach its tolerance raises
``SolveNotConverged`` (the gradient of an unconverged solve is not the
gradient of A^{-1} b); ``ctx.info`` / ``ctx.adjoint_info`` keep the solver's
report either way.
"""
from __future__ import annotations

import torch


class SolveNotConverged(RuntimeError):
    """A GMRES solve inside ``solve`` (forward or adjoint) stopped above its tolerance."""


def _require_converged(info, what):
    if not info["converged"]:
        raise SolveNotConverged(
            f"{what} GMRES stopped at relative residual {info['rel_residual']:.3e} after "
            f"{info['iterations']} iterations without reaching its tolerance")


class _Matvec(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, H, precision):
        ctx.H = H
        ctx.precision = precision
        return H.matvec(x.detach(), precision)

    @staticmethod
    def backward(ctx, g):
        return ctx.H.matvec(g.contiguous(), ctx.precision, transpose=True), None, None


class _Solve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, b, H, opts):
        ctx.H = H
        ctx.opts = opts
        x, info = H.gmres(b.detach(), **opts)
        ctx.info = info
        _require_converged(info, "forward")
        return x

    @staticmethod
    def backward(ctx, g):
        # the adjoint of a solve with A is a solve with A^T, and conversely
        opts = dict(ctx.opts)
        opts["transpose"] = not opts.get("transpose", False)
        lam, info = ctx.H.gmres(g.contiguous(), **opts)
        ctx.adjoint_info = info
        _require_converged(info, "adjoint")
        return lam, None, None


def matvec(H, x, precision="fp64"):
    """Differentiable y = A x (gradient w.r.t. the charges x)."""
    return _Matvec.apply(x, H, precision)


def solve(H, b, maxit=400, tol=1e-10, restart=30, precision="fp64", **kw):
    """Differentiable x = A^{-1} b (gradient w.r.t. the right-hand side b)."""
    opts = dict(maxit=maxit, tol=tol, restart=restart, precision=precision, **kw)
    return _Solve.apply(b, H, opts)
