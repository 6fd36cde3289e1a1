"""Kerr nonlinear solvers (fdfdpy/nonlinear_solvers.py:13-149) on the GPU.

born_solve  : fixed point E <- (A + Anl(E))^-1 b, refactoring each step
              (nonlinear_solvers.py:13-54).
newton_solve: Newton on f(E) = (A + Anl(E)) E - b with the Jacobian
              J11 = A + Anl + diag(dAde E), J12 = diag(conj(dAde) E),
              dAde = dnl_de omega^2 eps0' (nonlinear_solvers.py:57-149).
              The reference solves J11 d + J12 conj(d) = f as a real 2n x 2n
              system with PARDISO (solver_complex2real, linalg.py:152-186);
              here the complex factor of J11 preconditions real-inner-product
              GMRES on that real-linear system (solve_complex2real), so the
              Newton loop reuses the same GPU multifrontal engine.
Both keep E on the device between iterations; the Kerr terms are evaluated
on the device from the Nonlinearity definitions (nonlinearity.py:18-34).
"""
from __future__ import annotations

from copy import deepcopy

import numpy as np
import torch

from . import engine
from .constants import EPSILON_0, DEFAULT_TOL, DEFAULT_MAX_REFINE


def kerr_terms_device(simulation, E):
    """(eps_nl, dnl_de) on the device for a device field E (n,)."""
    dev = E.device
    n = E.numel()
    eps_nl = torch.zeros(n, dtype=torch.float64, device=dev)
    dnl_de = torch.zeros(n, dtype=torch.complex128, device=dev)
    eps_r = engine.as_f64(simulation.eps_r).reshape(-1)
    for nli in simulation.nonlinearity:
        if nli.nl_type != 'kerr':
            raise AssertionError("Only 'kerr' type nonlinearity is supported")
        region = engine.as_f64(nli.nl_region).reshape(-1)
        scale = (eps_r - 1) / (nli.eps_max - 1) if nli.eps_scale else 1.0
        eps_nl = eps_nl + 3 * nli.chi * region * (E.real ** 2 + E.imag ** 2) * scale
        dnl_de = dnl_de + 3 * nli.chi * region * torch.conj(E) * scale
    return eps_nl, dnl_de


def solve_complex2real(fac, J11_op, J12, f, tol=1e-12, max_iter=400, restart=60):
    """d with J11 d + J12 * conj(d) = f (J12 a diagonal as an (n,) vector).

    The operator d -> J11 d + J12 conj(d) is linear over the reals (the
    reference solves it as a real 2n x 2n system, linalg.py:152-186), so
    this is restarted GMRES in the real inner product Re<u, v> on C^n = R^2n,
    right-preconditioned by the complex factor of J11: d = J11^-1 y.  A plain
    fixed-point refinement with that factor diverges once |J12| is
    comparable to J11 (strong Kerr terms); GMRES does not need the
    contraction.  Every residual is formed in FP64 with the matrix-free
    J11.  Returns (d, relative residual, operator applications)."""
    fn = float(torch.linalg.vector_norm(f))
    if fn == 0.0:
        return torch.zeros_like(f), 0.0, 0

    def op(x):
        return J11_op.apply(x) + J12 * torch.conj(x)

    d = torch.zeros_like(f)
    r = f.clone()
    beta = fn
    rel, it = 1.0, 0
    while it < max_iter:
        m = min(restart, max_iter - it)
        V = torch.empty((m + 1,) + tuple(f.shape), dtype=f.dtype, device=f.device)
        Z = torch.empty((m,) + tuple(f.shape), dtype=f.dtype, device=f.device)
        V[0] = r / beta
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        k = 0
        for j in range(m):
            Z[j] = fac.apply_inverse(V[j])
            w = op(Z[j])
            it += 1
            Vj = V[:j + 1].reshape(j + 1, -1)
            for _ in range(2):  # classical Gram-Schmidt, twice, real inner product
                h = torch.real(Vj.conj() @ w.reshape(-1))
                w = w - (h.to(w.dtype) @ Vj).reshape(w.shape)
                H[:j + 1, j] += h.cpu().numpy()
            hn = float(torch.linalg.vector_norm(w))
            H[j + 1, j] = hn
            if hn > 0:
                V[j + 1] = w / hn
            for i in range(j):  # earlier rotations
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            den = np.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = (1.0, 0.0) if den == 0 else (H[j, j] / den, H[j + 1, j] / den)
            H[j, j] = cs[j] * H[j, j] + sn[j] * H[j + 1, j]
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            if abs(g[j + 1]) <= tol * fn or hn == 0:
                break
        y = np.linalg.solve(np.triu(H[:k, :k]), g[:k]) if k else np.zeros(0)
        yt = torch.as_tensor(y, dtype=torch.float64, device=f.device).to(f.dtype)
        d = d + (yt @ Z[:k].reshape(k, -1)).reshape(f.shape)
        r = f - op(d)
        prev, beta = beta, float(torch.linalg.vector_norm(r))
        rel = beta / fn
        if rel <= tol or beta == 0.0:
            break
        if beta > 0.5 * prev:
            # a whole cycle gained less than a factor of two on the FP64
            # residual: it has reached the rounding floor of the operator
            break
    return d, rel, it


def nl_eq_and_jac(simulation, averaging=True, Ex=None, Ey=None, Ez=None, compute_jac=True,
                  matrix_format='csr', precision=None):
    """f(E) and the Jacobian of the Kerr problem (nonlinear_solvers.py:117-149),
    device-resident: returns (f (n,), J11 operator, J12 (n,)) or f."""
    if simulation.pol != 'Ez':
        raise ValueError('Invalid polarization: {}'.format(str(simulation.pol)))
    omega = simulation.omega
    E = engine.as_c128(Ez).reshape(-1)
    eps_nl, dnl_de = kerr_terms_device(simulation, E)
    op_nl = simulation._op.with_terms(eps_add=eps_nl)
    b = engine.as_c128(simulation.src * 1j * omega).reshape(-1)
    fE = -op_nl.residual(E, b)                       # (A + Anl) E - b
    if not compute_jac:
        return fE
    dAde = dnl_de * (omega ** 2 * EPSILON_0 * simulation.L0)
    J11 = simulation._op.with_terms(eps_add=eps_nl, diag_add=dAde * E)
    J12 = torch.conj(dAde) * E
    return fE, J11, J12


def _start_field(simulation, Estart):
    if Estart is not None:
        return engine.as_c128(Estart).reshape(-1)
    if simulation.fields['Ez'] is None:
        simulation.solve_fields()
    return engine.as_c128(deepcopy(simulation.fields['Ez'])).reshape(-1)


def born_solve(simulation, Estart=None, conv_threshold=1e-10, max_num_iter=50, averaging=True):
    conv_array = np.zeros((max_num_iter, 1))
    if simulation.pol != 'Ez':
        raise ValueError('Invalid polarization: {}'.format(str(simulation.pol)))
    Ez = _start_field(simulation, Estart)
    prec = simulation.precision
    b = engine.as_c128(simulation.src * 1j * simulation.omega).reshape(-1)
    convergence = float('inf')
    for istep in range(max_num_iter):
        Eprev = Ez
        eps_nl, _ = kerr_terms_device(simulation, Eprev)
        op = simulation._op.with_terms(eps_add=eps_nl)
        fac = engine.Factor(engine.symbolic_for(simulation.Nx, simulation.Ny), prec).numeric(op)
        Ez = fac.solve(b, tol=DEFAULT_TOL[prec], max_iter=DEFAULT_MAX_REFINE[prec])
        convergence = float(torch.linalg.vector_norm(Ez - Eprev) / torch.linalg.vector_norm(Ez))
        conv_array[istep] = convergence
        if convergence < conv_threshold:
            break
    if convergence > conv_threshold:
        print("the simulation did not converge, reached {}".format(convergence))
    return _finish(simulation, Ez, conv_array, averaging)


def newton_solve(simulation, Estart=None, conv_threshold=1e-10, max_num_iter=50, averaging=True,
                 solver='pardiso', jac_solver='c2r', matrix_format='csr', lin_tol=1e-11):
    conv_array = np.zeros((max_num_iter, 1))
    if simulation.pol != 'Ez':
        raise ValueError('Invalid polarization: {}'.format(str(simulation.pol)))
    Ez = _start_field(simulation, Estart)
    prec = simulation.precision
    sym = engine.symbolic_for(simulation.Nx, simulation.Ny)
    convergence = float('inf')
    simulation.newton_stats = []
    for istep in range(max_num_iter):
        Eprev = Ez
        fx, J11, J12 = nl_eq_and_jac(simulation, Ez=Eprev)
        fac = engine.Factor(sym, prec).numeric(J11)
        Ediff, rel, its = solve_complex2real(fac, J11, J12, fx, tol=lin_tol)
        simulation.newton_stats.append({"linear_rel_residual": rel, "inner_iters": its})
        Ez = Eprev - Ediff
        convergence = float(torch.linalg.vector_norm(Ez - Eprev) / torch.linalg.vector_norm(Ez))
        conv_array[istep] = convergence
        if convergence < conv_threshold:
            break
    if convergence > conv_threshold:
        print("the simulation did not converge, reached {}".format(convergence))
    return _finish(simulation, Ez, conv_array, averaging)


def _finish(simulation, Ez, conv_array, averaging):
    """Final solve with the converged eps_nl (nonlinear_solvers.py:106-107)."""
    simulation.compute_nl(Ez.cpu().numpy().reshape(simulation.Nx, simulation.Ny))
    (Hx, Hy, Ez_out) = simulation.solve_fields(include_nl=True, averaging=averaging)
    return (Hx, Hy, Ez_out, conv_array)
