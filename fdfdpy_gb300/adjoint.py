"""Differentiable FDFD solve (no counterpart in the reference, which has no
derivative with respect to eps; the operator derivative follows from
fdfdpy/linalg.py:53-54, 66: dA/d eps_p = omega^2 eps0' e_p e_p^T for Ez).

``solve_ez(eps_r, src, ...)`` returns the Ez field as a complex128 tensor
and is differentiable with respect to eps_r and src.  The backward pass is
one transposed solve on the forward factor -- A^T = P A P^-1 with
P = diag(sxf syf), so the factor of A serves A^T -- followed by the
gradient kernel (K9):

    lambda = A^-T conj(g),     dL/d eps_r = -omega^2 eps0' Re(lambda E),
    dL/d src = conj(1j omega lambda)  (Re(...) for a real src),

with g the incoming gradient in torch's convention for complex tensors.
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine
from .constants import DEFAULT_LENGTH_SCALE, DEFAULT_TOL, DEFAULT_MAX_REFINE


class _EzSolve(torch.autograd.Function):

    @staticmethod
    def forward(ctx, eps_r, src, omega, dl, NPML, L0, precision, tol):
        Nx, Ny = eps_r.shape
        op = engine.DeviceOperator(omega, eps_r.detach(), Nx * dl, Ny * dl, NPML, "Ez", L0)
        fac = engine.Factor(engine.symbolic_for(Nx, Ny), precision).numeric(op)
        b = (1j * omega) * engine.as_c128(src.detach()).reshape(-1)
        E = fac.solve(b, tol=tol, max_iter=DEFAULT_MAX_REFINE[precision])
        ctx.fac, ctx.op, ctx.omega, ctx.tol, ctx.precision = fac, op, omega, tol, precision
        ctx.src_complex = src.is_complex()
        ctx.save_for_backward(E)
        return E.reshape(Nx, Ny)

    @staticmethod
    def backward(ctx, gE):
        (E,) = ctx.saved_tensors
        Nx, Ny = gE.shape
        rhs = torch.conj(engine.as_c128(gE)).reshape(-1).contiguous()
        lam = ctx.fac.solve(rhs, transpose=True, tol=ctx.tol, max_iter=DEFAULT_MAX_REFINE[ctx.precision])
        g_eps = ctx.op.grad_eps(lam, E).reshape(Nx, Ny) if ctx.needs_input_grad[0] else None
        g_src = None
        if ctx.needs_input_grad[1]:
            c = (1j * ctx.omega) * lam
            g_src = torch.conj(c).reshape(Nx, Ny) if ctx.src_complex else c.real.reshape(Nx, Ny)
        return g_eps, g_src, None, None, None, None, None, None


def solve_ez(eps_r: torch.Tensor, src: torch.Tensor, omega: float, dl: float, NPML,
             L0: float = DEFAULT_LENGTH_SCALE, precision: str = "c128", tol: float | None = None):
    """Ez = A(eps_r)^-1 (1j omega src) on the GPU, differentiable in eps_r
    (float64) and src (real or complex)."""
    tol = DEFAULT_TOL[precision] if tol is None else tol
    return _EzSolve.apply(eps_r, src, float(omega), float(dl), [int(NPML[0]), int(NPML[1])], float(L0),
                          precision, tol)
