"""Differentiable FDFD solves (no counterpart in the reference, which has no
derivative with respect to eps; the operator derivatives follow from
fdfdpy/linalg.py:52-93 and the Kerr terms from fdfdpy/nonlinearity.py:18-34).

``solve(eps_r, src, omega, dl, NPML, pol)`` returns the primary field (Ez or
Hz) as a complex128 tensor, differentiable with respect to eps_r and src.
The backward pass is one transposed solve on the forward factor --
A^T = P A P^-1 with P = diag(sxf syf), so the factor of A serves A^T --
followed by the gradient kernel (K9, fdfd_adjoint_grad_eps):

    lambda = A^-T conj(g),     dL/d eps_r = K9(lambda, E),
    dL/d src = Re(1j omega lambda)  (conj(1j omega lambda) for a complex src),

with g the incoming gradient in torch's convention for complex tensors.

``solve_kerr_ez(...)`` is the same for the Kerr-nonlinear Ez problem solved
by Newton (nonlinear_solvers.newton_device).  At the converged field E,
F(E, eps) = (A + diag(w eps_nl(E, eps))) E - b = 0 with w = omega^2 eps0';
its derivative in E is the real-linear Newton Jacobian d -> J11 d +
J12 conj(d), so the adjoint field solves the real-linear system

    J11^T lambda + conj(J12) conj(lambda) = conj(g)

(GMRES in the real inner product, preconditioned by the transposed J11
factor of the forward Newton loop), and
    dL/d eps_r = -w Re(lambda E) (1 + dnl_deps),  dL/d src as above.

``Simulation.solve_fields_torch`` and ``design_step`` put these behind the
Simulation API for optimisation loops over a design region
(Simulation.init_design_region, simulation.py:344-369).
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine
from .constants import DEFAULT_LENGTH_SCALE, DEFAULT_TOL, DEFAULT_MAX_REFINE, EPSILON_0


def _src_grad(lam, omega, src_complex, shape):
    c = (1j * omega) * lam
    return torch.conj(c).reshape(shape) if src_complex else c.real.reshape(shape)


class _FieldSolve(torch.autograd.Function):

    @staticmethod
    def forward(ctx, eps_r, src, omega, dl, NPML, L0, pol, precision, tol):
        Nx, Ny = eps_r.shape
        op = engine.DeviceOperator(omega, eps_r.detach(), Nx * dl, Ny * dl, NPML, pol, L0)
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
        g_src = _src_grad(lam, ctx.omega, ctx.src_complex, (Nx, Ny)) if ctx.needs_input_grad[1] else None
        return g_eps, g_src, None, None, None, None, None, None, None


def solve(eps_r: torch.Tensor, src: torch.Tensor, omega: float, dl: float, NPML, pol: str = "Ez",
          L0: float = DEFAULT_LENGTH_SCALE, precision: str = "c128", tol: float | None = None):
    """Primary field (Ez or Hz) = A(eps_r)^-1 (1j omega src) on the GPU,
    differentiable in eps_r (float64) and src (real or complex)."""
    tol = DEFAULT_TOL[precision] if tol is None else tol
    return _FieldSolve.apply(eps_r, src, float(omega), float(dl), [int(NPML[0]), int(NPML[1])], float(L0), pol,
                             precision, tol)


def solve_ez(eps_r: torch.Tensor, src: torch.Tensor, omega: float, dl: float, NPML,
             L0: float = DEFAULT_LENGTH_SCALE, precision: str = "c128", tol: float | None = None):
    """Ez = A(eps_r)^-1 (1j omega src) on the GPU, differentiable in eps_r
    (float64) and src (real or complex)."""
    return solve(eps_r, src, omega, dl, NPML, "Ez", L0, precision, tol)


class _KerrSolve(torch.autograd.Function):

    @staticmethod
    def forward(ctx, eps_r, src, omega, dl, NPML, L0, nonlinearities, precision, conv_threshold, max_num_iter):
        from .nonlinear_solvers import KerrTerms, newton_device
        Nx, Ny = eps_r.shape
        op = engine.DeviceOperator(omega, eps_r.detach(), Nx * dl, Ny * dl, NPML, "Ez", L0)
        b = (1j * omega) * engine.as_c128(src.detach()).reshape(-1)
        tol = DEFAULT_TOL[precision]
        E0 = engine.Factor(engine.symbolic_for(Nx, Ny), precision).numeric(op).solve(
            b, tol=tol, max_iter=DEFAULT_MAX_REFINE[precision])
        kerr = KerrTerms(omega, L0, op.eps, nonlinearities)
        stats = {}
        E, conv, fac = newton_device(op, b, kerr, E0, precision, conv_threshold, max_num_iter, stats=stats)
        ctx.conv = conv
        ctx.fac, ctx.op, ctx.kerr, ctx.omega, ctx.L0 = fac, op, kerr, omega, L0
        ctx.src_complex = src.is_complex()
        ctx.save_for_backward(E)
        return E.reshape(Nx, Ny)

    @staticmethod
    def backward(ctx, gE):
        from .nonlinear_solvers import solve_complex2real
        (E,) = ctx.saved_tensors
        Nx, Ny = gE.shape
        t = ctx.kerr(E, eps_nl=True, jac=True, deps=True)
        J11 = ctx.op.with_terms(eps_add=t['eps_nl'], diag_add=t['jac_diag'])
        rhs = torch.conj(engine.as_c128(gE)).reshape(-1).contiguous()
        lam, rel, _ = solve_complex2real(ctx.fac, J11, torch.conj(t['jac_off']), rhs, tol=1e-12, transpose=True)
        g_eps = None
        if ctx.needs_input_grad[0]:
            # K9 gives -w Re(lambda E); the Kerr term adds the eps dependence of eps_nl
            g_eps = (ctx.op.grad_eps(lam, E) * (1.0 + t['dnl_deps'])).reshape(Nx, Ny)
        g_src = _src_grad(lam, ctx.omega, ctx.src_complex, (Nx, Ny)) if ctx.needs_input_grad[1] else None
        return g_eps, g_src, None, None, None, None, None, None, None, None


def solve_kerr_ez(eps_r: torch.Tensor, src: torch.Tensor, omega: float, dl: float, NPML, chi: float,
                  nl_region, eps_scale: bool = False, eps_max: float | None = None,
                  L0: float = DEFAULT_LENGTH_SCALE, precision: str = "c128", conv_threshold: float = 1e-12,
                  max_num_iter: int = 50):
    """Ez of the Kerr-nonlinear problem (chi in m^2/V^2 as given to
    Simulation.add_nl, which divides it by L0^2) by Newton on the GPU,
    differentiable in eps_r and src through the adjoint of the Newton
    Jacobian at the converged field."""
    from .nonlinearity import Nonlinearity
    nl = [Nonlinearity(chi / L0 ** 2, np.asarray(nl_region, dtype=np.float64), 'kerr', eps_scale, eps_max)]
    return _KerrSolve.apply(eps_r, src, float(omega), float(dl), [int(NPML[0]), int(NPML[1])], float(L0), nl,
                            precision, float(conv_threshold), int(max_num_iter))


def secondary_fields(X, eps_r, omega, dl, NPML, pol, L0=DEFAULT_LENGTH_SCALE, averaging=True):
    """The two secondary fields of simulation.py:129-175 from the primary
    field X (Nx, Ny), as differentiable torch expressions of X (and of eps_r
    for Hz): Ez -> (Hx, Hy), Hz -> (Ex, Ey)."""
    Nx, Ny = X.shape
    op = engine.DeviceOperator(omega, eps_r.detach() if isinstance(eps_r, torch.Tensor) else eps_r,
                               Nx * dl, Ny * dl, NPML, pol, L0)
    isxb, isyb = op.inv_s[1], op.inv_s[3]
    dxb = (X - torch.roll(X, 1, 0)) * (isxb[:, None] * (Nx / (Nx * dl)))
    dyb = (X - torch.roll(X, 1, 1)) * (isyb[None, :] * (Ny / (Ny * dl)))
    if pol == "Ez":
        mu0 = 1.25663706e-6 * L0
        return -1 / 1j / omega / mu0 * dyb, 1 / 1j / omega / mu0 * dxb
    e = EPSILON_0 * L0 * (eps_r if isinstance(eps_r, torch.Tensor) else torch.as_tensor(eps_r, device=X.device))
    ex = (torch.roll(e, 1, 0) + e) / 2 if averaging else e
    ey = (torch.roll(e, 1, 1) + e) / 2 if averaging else e
    return 1 / 1j / omega * (dyb / ey), -1 / 1j / omega * (dxb / ex)


def design_step(sim, design_region, objective, eps_m, step=1.0, eps=None):
    """One projected gradient-ascent step of the objective over the design
    region of a Simulation (the eps_r that init_design_region,
    simulation.py:344-369, initialises): J = objective(fields) with fields
    from Simulation.solve_fields_torch, eps_r[region] += step * dJ/deps
    scaled to at most one unit of permittivity, clipped to [1, eps_m].
    Returns (J, gradient over the region) and updates sim.eps_r."""
    e = torch.tensor(np.asarray(sim.eps_r if eps is None else eps, dtype=np.float64), device=engine.device(),
                     requires_grad=True)
    J = objective(sim.solve_fields_torch(e))
    J.backward()
    g = e.grad.detach()
    mask = torch.as_tensor(np.asarray(design_region) != 0, device=g.device)
    gm = torch.where(mask, g, torch.zeros_like(g))
    scale = float(gm.abs().max())
    new = e.detach() + (step / scale if scale > 0 else 0.0) * gm
    new = torch.where(mask, new.clamp(1.0, float(eps_m)), e.detach())
    sim.eps_r = new.cpu().numpy()
    return float(J.detach()), gm
