"""Kerr nonlinear solvers (fdfdpy/nonlinear_solvers.py:13-149) on the GPU.

born_solve  : fixed point E <- (A + Anl(E))^-1 b (nonlinear_solvers.py:13-54).
newton_solve: Newton on f(E) = (A + Anl(E)) E - b with the Jacobian
              J11 = A + Anl + diag(dAde E), J12 = diag(conj(dAde) E),
              dAde = dnl_de omega^2 eps0' (nonlinear_solvers.py:57-149).
              The reference solves J11 d + J12 conj(d) = f as a real 2n x 2n
              system with PARDISO (solver_complex2real, linalg.py:152-186);
              here the complex factor of J11 preconditions real-inner-product
              GMRES on that real-linear system (solve_complex2real), so the
              Newton loop reuses the same GPU multifrontal engine.

Factor reuse: neither loop refactors every iteration.  The factor of the
first iterate's operator (Born: A + Anl; Newton: J11) preconditions
Jacobian-free GMRES on the current iterate's operator, applied matrix-free
in FP64; the operator is refactored only when that GMRES needs more than
`max_inner` factor applications (the iterate has moved far from the
factored one).  Both keep E on the device between iterations; the Kerr
terms come from one kernel per nonlinearity (fdfd_kerr_assemble, K1-NL).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import engine
from . import _native as N
from .constants import DEFAULT_TOL, DEFAULT_MAX_REFINE


class KerrTerms:
    """The Kerr nonlinearities of a simulation as device data: for each, chi
    (already divided by L0^2, simulation.py:72), the region and eps scaling
    (nonlinearity.py:18-34), evaluated by fdfd_kerr_assemble."""

    def __init__(self, omega, L0, eps_r_dev, nonlinearities):
        self.omega, self.L0 = float(omega), float(L0)
        self.eps_r = eps_r_dev.reshape(-1)
        self.items = []
        for nli in nonlinearities:
            if nli.nl_type != 'kerr':
                raise AssertionError("Only 'kerr' type nonlinearity is supported")
            region = engine.as_f64(nli.nl_region).reshape(-1)
            self.items.append((float(nli.chi), region, bool(nli.eps_scale),
                               float(nli.eps_max) if nli.eps_scale else 0.0))

    @classmethod
    def of(cls, simulation):
        return cls(simulation.omega, simulation.L0, simulation._op.eps, simulation.nonlinearity)

    def __call__(self, E, eps_nl=True, jac=False, deps=False, de=False):
        """Device tensors {'eps_nl', 'jac_diag', 'jac_off', 'dnl_deps',
        'dnl_de'} (the requested ones) for the device field E (n,)."""
        E = engine.as_c128(E).reshape(-1)
        n = E.numel()
        dev = E.device
        out = {}
        if eps_nl:
            out['eps_nl'] = torch.zeros(n, dtype=torch.float64, device=dev)
        if deps:
            out['dnl_deps'] = torch.zeros(n, dtype=torch.float64, device=dev)
        if de:
            out['dnl_de'] = torch.zeros(n, dtype=torch.complex128, device=dev)
        if jac:
            out['jac_diag'] = torch.zeros(n, dtype=torch.complex128, device=dev)
            out['jac_off'] = torch.zeros(n, dtype=torch.complex128, device=dev)
        p = lambda k: engine._ptr(out.get(k))  # noqa: E731
        for idx, (chi, region, scale, eps_max) in enumerate(self.items):
            N.call("fdfd_kerr_assemble", n, engine._ptr(E), engine._ptr(self.eps_r), engine._ptr(region), chi,
                   int(scale), eps_max, self.omega, self.L0, int(idx > 0), p('eps_nl'), p('dnl_deps'),
                   p('dnl_de'), p('jac_diag'), p('jac_off'), engine.stream_ptr())
        return out


def kerr_terms_device(simulation, E):
    """(eps_nl, dnl_de) on the device for a device field E (n,)."""
    t = KerrTerms.of(simulation)(E, eps_nl=True, de=True)
    return t['eps_nl'], t['dnl_de']


def solve_complex2real(fac, J11_op, J12, f, tol=1e-12, max_iter=400, restart=60, transpose=False):
    """d with J11 d + J12 * conj(d) = f (J12 a diagonal as an (n,) vector);
    with transpose, J11^T d + J12 * conj(d) = f.

    The operator d -> J11 d + J12 conj(d) is linear over the reals (the
    reference solves it as a real 2n x 2n system, linalg.py:152-186), so
    this is restarted GMRES in the real inner product Re<u, v> on C^n = R^2n,
    right-preconditioned by the complex factor of J11 (or of a nearby
    operator): d = J11^-1 y.  A plain fixed-point refinement with that
    factor diverges once |J12| is comparable to J11 (strong Kerr terms);
    GMRES does not need the contraction.  Every residual is formed in FP64
    with the matrix-free J11.  Returns (d, relative residual, operator
    applications)."""
    fn = float(torch.linalg.vector_norm(f))
    if fn == 0.0:
        return torch.zeros_like(f), 0.0, 0

    def op(x):
        return J11_op.apply(x, transpose=transpose) + J12 * torch.conj(x)

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
            Z[j] = fac.apply_inverse(V[j], transpose=transpose)
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
    b = engine.as_c128(simulation.src * 1j * simulation.omega).reshape(-1)
    return _f_and_jac(simulation._op, b, KerrTerms.of(simulation), engine.as_c128(Ez).reshape(-1), compute_jac)


def _f_and_jac(op_lin, b, kerr, E, compute_jac=True):
    t = kerr(E, eps_nl=True, jac=compute_jac)
    op_nl = op_lin.with_terms(eps_add=t['eps_nl'])
    fE = -op_nl.residual(E, b)                       # (A + Anl) E - b
    if not compute_jac:
        return fE
    J11 = op_lin.with_terms(eps_add=t['eps_nl'], diag_add=t['jac_diag'])
    return fE, J11, t['jac_off']


def _rel_change(E, Eprev):
    return float(torch.linalg.vector_norm(E - Eprev) / torch.linalg.vector_norm(E))


def newton_device(op_lin, b, kerr, E0, precision, conv_threshold=1e-10, max_num_iter=50, lin_tol=1e-11,
                  reuse_factor=True, max_inner=30, stats=None):
    """Newton iterations from the device field E0; returns (E, conv_array,
    factor) with the factor last used (of J11 at some iterate).  The factor
    is reused while it keeps preconditioning well: an iteration whose reuse
    attempt ran out of inner iterations refactors, and so does the next one
    (the iterate is moving fast) until an iteration converges with the
    factor in at most max_inner / 2 applications."""
    sym = engine.symbolic_for(op_lin.Nx, op_lin.Ny)
    conv_array = np.zeros((max_num_iter, 1))
    E = E0
    fac = None
    stats = {} if stats is None else stats
    stats.update(factorizations=0, inner=[], linear_rel_residual=[])
    convergence = float('inf')
    trust = False        # the factor in hand preconditioned the last solve well
    for istep in range(max_num_iter):
        Eprev = E
        fx, J11, J12 = _f_and_jac(op_lin, b, kerr, Eprev)
        rel, its, d = 1.0, 0, None
        if fac is not None and reuse_factor and trust:
            d, rel, its = solve_complex2real(fac, J11, J12, fx, tol=lin_tol, max_iter=max_inner)
        if d is None or rel > max(lin_tol, 1e-9):
            reuse_failed = d is not None
            fac = engine.Factor(sym, precision).numeric(J11)
            stats['factorizations'] += 1
            d, rel, its2 = solve_complex2real(fac, J11, J12, fx, tol=lin_tol)
            its += its2
            # after a failed reuse the iterate is moving fast: refactor next time too
            trust = not reuse_failed and its2 <= max_inner // 2
        else:
            trust = its <= max_inner // 2
        stats['inner'].append(its)
        stats['linear_rel_residual'].append(rel)
        E = Eprev - d
        convergence = _rel_change(E, Eprev)
        conv_array[istep] = convergence
        if not convergence >= conv_threshold:   # NaN ends the loop too
            break
    if not convergence <= conv_threshold:
        print("the simulation did not converge, reached {}".format(convergence))
    return E, conv_array, fac


def born_device(op_lin, b, kerr, E0, precision, conv_threshold=1e-10, max_num_iter=50, reuse_factor=True,
                max_inner=30, stats=None):
    """Born iterations from the device field E0; returns (E, conv_array,
    factor)."""
    sym = engine.symbolic_for(op_lin.Nx, op_lin.Ny)
    conv_array = np.zeros((max_num_iter, 1))
    E = E0
    fac = None
    stats = {} if stats is None else stats
    stats.update(factorizations=0, inner=[])
    tol = DEFAULT_TOL[precision]
    convergence = float('inf')
    for istep in range(max_num_iter):
        Eprev = E
        op = op_lin.with_terms(eps_add=kerr(Eprev)['eps_nl'])
        E = None
        if fac is not None and reuse_factor:
            try:
                E = fac.solve(b, op=op, method='gmres', tol=tol, max_iter=max_inner, raise_on_fail=True)
            except N.NotConverged:
                E = None
        if E is None:
            fac = engine.Factor(sym, precision).numeric(op)
            stats['factorizations'] += 1
            E = fac.solve(b, op=op, tol=tol, max_iter=DEFAULT_MAX_REFINE[precision])
        stats['inner'].append(fac.stats()['refine_iters'])
        convergence = _rel_change(E, Eprev)
        conv_array[istep] = convergence
        if not convergence >= conv_threshold:
            break
    if not convergence <= conv_threshold:
        print("the simulation did not converge, reached {}".format(convergence))
    return E, conv_array, fac


def _start_field(simulation, Estart):
    if Estart is not None:
        return engine.as_c128(Estart).reshape(-1)
    if simulation.fields['Ez'] is None:
        simulation.solve_fields()
    return engine.as_c128(simulation.fields['Ez']).reshape(-1)


def _rhs(simulation):
    return engine.as_c128(simulation.src * 1j * simulation.omega).reshape(-1)


def born_solve(simulation, Estart=None, conv_threshold=1e-10, max_num_iter=50, averaging=True,
               reuse_factor=True):
    if simulation.pol != 'Ez':
        raise ValueError('Invalid polarization: {}'.format(str(simulation.pol)))
    Ez = _start_field(simulation, Estart)
    kerr = KerrTerms.of(simulation)
    simulation.nl_stats = {}
    Ez, conv_array, fac = born_device(simulation._op, _rhs(simulation), kerr, Ez, simulation.precision,
                                      conv_threshold, max_num_iter, reuse_factor, stats=simulation.nl_stats)
    return _finish(simulation, Ez, conv_array, averaging, kerr, fac)


def newton_solve(simulation, Estart=None, conv_threshold=1e-10, max_num_iter=50, averaging=True,
                 solver='pardiso', jac_solver='c2r', matrix_format='csr', lin_tol=1e-11, reuse_factor=True):
    if simulation.pol != 'Ez':
        raise ValueError('Invalid polarization: {}'.format(str(simulation.pol)))
    Ez = _start_field(simulation, Estart)
    kerr = KerrTerms.of(simulation)
    simulation.nl_stats = {}
    Ez, conv_array, fac = newton_device(simulation._op, _rhs(simulation), kerr, Ez, simulation.precision,
                                        conv_threshold, max_num_iter, lin_tol, reuse_factor,
                                        stats=simulation.nl_stats)
    simulation.newton_stats = [{"linear_rel_residual": r, "inner_iters": i}
                               for r, i in zip(simulation.nl_stats['linear_rel_residual'],
                                               simulation.nl_stats['inner'])]
    return _finish(simulation, Ez, conv_array, averaging, kerr, fac)


def _finish(simulation, Ez, conv_array, averaging, kerr, fac=None):
    """The final linear solve with the converged eps_nl
    (nonlinear_solvers.py:106-107, simulation.py:124-126) and the fields;
    the Kerr terms are evaluated on the device (the simulation's eps_nl,
    dnl_de and dnl_deps attributes receive host copies)."""
    t = kerr(Ez, eps_nl=True, deps=True, de=True)
    simulation._set_nl_device(t['eps_nl'])
    simulation.dnl_de, simulation.dnl_deps = (a.reshape(simulation.Nx, simulation.Ny)
                                              for a in engine.to_host(t['dnl_de'], t['dnl_deps']))
    (Hx, Hy, Ez_out) = simulation.solve_fields(include_nl=True, averaging=averaging, preconditioner=fac)
    return (Hx, Hy, Ez_out, conv_array)
