"""CPU oracle for the FDFD hot path -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import it.  The GPU engine (``fdfdpy_gb300``) never calls into it.

It restates, in numpy/scipy, the algorithm of fdfdpy's hot path:

* ``sfactor``          -- fdfdpy/pml.py:7-39 (sig_w, S, create_sfactor)
* ``inv_sfactors``     -- the 1/s broadcast of S_create, pml.py:64-75
* ``stencil``          -- construct_A, fdfdpy/linalg.py:41-107, written as
                          the five diagonals of the periodic 5-point operator
* ``construct_A``      -- canonical CSR (sorted rows) of that operator
* ``derivs``           -- the S-scaled derivative operators, linalg.py:59-62
* ``solve``            -- solver_direct(solver='scipy'), linalg.py:122-149
                          (SuperLU through scipy.sparse.linalg.spsolve)
* ``fields``           -- field recovery, fdfdpy/simulation.py:129-175
* ``flux_probe``       -- fdfdpy/simulation.py:260-315

Complex products are written out as real arithmetic in the order scipy's
sparsetools complex type uses ((ar*br - ai*bi), (ar*bi + ai*br)), so the
oracle reproduces the reference's CSR values to the last bit or within an
ulp.  The oracle is pinned against golden vectors produced by running the
reference itself (tests/golden/make_golden.py) -- see
tests/test_oracle_golden.py.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

EPSILON_0 = 8.85418782e-12          # fdfdpy/constants.py:3
MU_0 = 1.25663706e-6                # fdfdpy/constants.py:4
C_0 = np.sqrt(1 / EPSILON_0 / MU_0)  # fdfdpy/constants.py:5
ETA_0 = np.sqrt(MU_0 / EPSILON_0)   # fdfdpy/constants.py:6


# ---- PML (fdfdpy/pml.py) ---------------------------------------------------
def _sig_w(l, dw, m=4, lnR=-12):
    sig_max = -(m + 1) * lnR / (2 * ETA_0 * dw)   # pml.py:10
    return sig_max * (l / dw) ** m                  # pml.py:11


def _s_value(l, dw, omega, L0):
    return 1 - 1j * _sig_w(l, dw) / (omega * EPSILON_0 * L0)   # pml.py:17


def sfactor(wlen, L0, s, omega, Nw, Nw_pml):
    """Stretch factors s(i) of one axis on the 'f' or 'b' grid (pml.py:20-39).

    A scalar loop over the Nw cells (O(Nw), small) so that every value goes
    through the same float64 scalar operations as the reference."""
    out = np.ones(Nw, dtype=np.complex128)
    if Nw_pml < 1:
        return out
    hw = np.float64(wlen) / Nw
    dw = Nw_pml * hw
    half = 0.5 if s == 'f' else 1
    for i in range(Nw):
        if i <= Nw_pml:
            out[i] = _s_value(hw * (Nw_pml - i + half), dw, omega, L0)
        elif i > Nw - Nw_pml:
            out[i] = _s_value(hw * (i - (Nw - Nw_pml) - half), dw, omega, L0)
    return out


def inv_sfactors(omega, L0, Nx, Ny, NPML, xlen, ylen):
    """The four 1-D vectors 1/s (x f, x b, y f, y b) that S_create spreads
    over the grid (pml.py:57-75)."""
    return (1 / sfactor(xlen, L0, 'f', omega, Nx, NPML[0]),
            1 / sfactor(xlen, L0, 'b', omega, Nx, NPML[0]),
            1 / sfactor(ylen, L0, 'f', omega, Ny, NPML[1]),
            1 / sfactor(ylen, L0, 'b', omega, Ny, NPML[1]))


# ---- complex helpers on (re, im) float arrays --------------------------------
def _mul(a, b):
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def _scale(a, s):
    return (a[0] * s, a[1] * s)


def _add(a, b):
    return (a[0] + b[0], a[1] + b[1])


def _ri(z):
    z = np.asarray(z, dtype=np.complex128)
    return (z.real.copy(), z.imag.copy())


def grid_average(a, w):
    """(roll(a, 1, axis) + a) / 2 (fdfdpy/linalg.py:16-22)."""
    ax = {'x': 0, 'y': 1}[w]
    return (np.roll(a, 1, axis=ax) + a) / 2


def _spacing(Nx, Ny, xlen, ylen):
    # dL (linalg.py:25-33): (xrange[1]-xrange[0]) / N
    L = np.array([xlen, ylen], dtype=np.float64)
    d = L / np.array([Nx, Ny])
    return d[0], d[1]


# ---- operator (fdfdpy/linalg.py:41-107) -------------------------------------
def stencil(omega, xlen, ylen, eps_r, NPML, pol, L0, averaging=True, eps_add=None, diag_add=None):
    """Five (Nx, Ny) complex128 arrays: centre, (i-1), (i+1), (j-1), (j+1)
    coefficients of each row of the operator."""
    eps_r = np.asarray(eps_r, dtype=np.float64)
    Nx, Ny = eps_r.shape
    dx, dy = _spacing(Nx, Ny, xlen, ylen)
    vx, vy = 1 / dx, 1 / dy
    EPS0_ = EPSILON_0 * L0
    MU0_ = MU_0 * L0
    isxf, isxb, isyf, isyb = inv_sfactors(omega, L0, Nx, Ny, NPML, xlen, ylen)
    a = _ri(isxf[:, None] * np.ones((1, Ny)))
    ay = _ri(np.ones((Nx, 1)) * isyf[None, :])
    b0 = _ri(isxb[:, None] * np.ones((1, Ny)))
    b1 = _ri(np.roll(isxb, -1)[:, None] * np.ones((1, Ny)))
    by0 = _ri(np.ones((Nx, 1)) * isyb[None, :])
    by1 = _ri(np.ones((Nx, 1)) * np.roll(isyb, -1)[None, :])
    fxp, fxn = _scale(a, vx), _scale(a, -vx)
    fyp, fyn = _scale(ay, vy), _scale(ay, -vy)
    bx0p, bx0n, bx1p, bx1n = _scale(b0, vx), _scale(b0, -vx), _scale(b1, vx), _scale(b1, -vx)
    by0p, by0n, by1p, by1n = _scale(by0, vy), _scale(by0, -vy), _scale(by1, vy), _scale(by1, -vy)
    if pol == 'Ez':
        invmu = 1. / MU0_
        fxp, fxn, fyp, fyn = (_scale(t, invmu) for t in (fxp, fxn, fyp, fyn))
        xm, xp = _mul(fxn, bx0n), _mul(fxp, bx1p)
        ym, yp = _mul(fyn, by0n), _mul(fyp, by1p)
        cx = _add(_mul(fxn, bx0p), _mul(fxp, bx1n))
        cy = _add(_mul(fyn, by0p), _mul(fyp, by1n))
        c = _add(cx, cy)
        c = (c[0] + omega ** 2 * (EPS0_ * eps_r), c[1])
    elif pol == 'Hz':
        E = EPS0_ * eps_r
        if averaging:
            ex, ey = grid_average(E, 'x'), grid_average(E, 'y')
        else:
            ex, ey = E, E
        tx0, ty0 = 1 / ex, 1 / ey
        tx1, ty1 = np.roll(tx0, -1, axis=0), np.roll(ty0, -1, axis=1)
        gxn, gxp = _scale(fxn, tx0), _scale(fxp, tx1)
        gyn, gyp = _scale(fyn, ty0), _scale(fyp, ty1)
        xm, xp = _mul(gxn, bx0n), _mul(gxp, bx1p)
        ym, yp = _mul(gyn, by0n), _mul(gyp, by1p)
        cx = _add(_mul(gxn, bx0p), _mul(gxp, bx1n))
        cy = _add(_mul(gyn, by0p), _mul(gyp, by1n))
        c = _add(cx, cy)
        c = (c[0] + omega ** 2 * MU0_, c[1])
    else:
        raise ValueError("pol must be one of 'Ez', 'Hz'")
    if eps_add is not None:
        c = (c[0] + omega ** 2 * EPSILON_0 * L0 * np.asarray(eps_add, dtype=np.float64), c[1])
    if diag_add is not None:
        c = _add(c, _ri(diag_add))
    to_c = lambda t: t[0] + 1j * t[1]
    return to_c(c), to_c(xm), to_c(xp), to_c(ym), to_c(yp)


def _neighbours(Nx, Ny):
    i, j = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing='ij')
    k = i * Ny + j
    return (k, ((i - 1) % Nx) * Ny + j, ((i + 1) % Nx) * Ny + j,
            i * Ny + (j - 1) % Ny, i * Ny + (j + 1) % Ny)


def construct_A(omega, xlen, ylen, eps_r, NPML, pol, L0, averaging=True, eps_add=None,
                diag_add=None):
    """Canonical CSR (indices sorted within rows, int32 indices) of the
    operator of construct_A (fdfdpy/linalg.py:41-107).  Requires Nx, Ny >= 3
    (then the five columns of every row are distinct)."""
    eps_r = np.asarray(eps_r, dtype=np.float64)
    Nx, Ny = eps_r.shape
    vals = np.stack([v.reshape(-1) for v in stencil(omega, xlen, ylen, eps_r, NPML, pol, L0,
                                                      averaging, eps_add, diag_add)], axis=1)
    cols = np.stack([c.reshape(-1) for c in _neighbours(Nx, Ny)], axis=1)
    order = np.argsort(cols, axis=1, kind='stable')
    cols = np.take_along_axis(cols, order, axis=1).astype(np.int32)
    vals = np.take_along_axis(vals, order, axis=1)
    n = Nx * Ny
    indptr = (5 * np.arange(n + 1)).astype(np.int32)
    return sp.csr_matrix((vals.reshape(-1), cols.reshape(-1), indptr), shape=(n, n))


def derivs(omega, xlen, ylen, Nx, Ny, NPML, L0):
    """Dxf, Dxb, Dyf, Dyb with their S factors (linalg.py:59-62), canonical CSR."""
    dx, dy = _spacing(Nx, Ny, xlen, ylen)
    vx, vy = 1 / dx, 1 / dy
    isxf, isxb, isyf, isyb = inv_sfactors(omega, L0, Nx, Ny, NPML, xlen, ylen)
    k, xm, xp, ym, yp = (c.reshape(-1) for c in _neighbours(Nx, Ny))
    ax = lambda v: np.repeat(v, Ny)
    ay = lambda v: np.tile(v, Nx)
    out = {}
    for name, s, v, other in (('Dxf', ax(isxf), vx, xp), ('Dxb', ax(isxb), vx, xm),
                              ('Dyf', ay(isyf), vy, yp), ('Dyb', ay(isyb), vy, ym)):
        sr = _ri(s)
        if name.endswith('f'):
            dval, oval = _scale(sr, -v), _scale(sr, v)
        else:
            dval, oval = _scale(sr, v), _scale(sr, -v)
        rows = np.concatenate([k, k])
        cols = np.concatenate([k, other])
        data = np.concatenate([dval[0] + 1j * dval[1], oval[0] + 1j * oval[1]])
        M = sp.csr_matrix((data, (rows, cols)), shape=(k.size, k.size))
        M.sort_indices()
        out[name] = M
    return out


# ---- solve (fdfdpy/linalg.py:122-149) ---------------------------------------
def solve(A, b):
    """x = A^-1 b by SuperLU (scipy spsolve), the reference's solver='scipy'
    branch; an all-zero b returns float zeros (linalg.py:128-129)."""
    b = np.asarray(b).astype(np.complex128).reshape(-1)
    if not b.any():
        return np.zeros(b.shape)
    return spl.spsolve(A.tocsc(), b)


def refine(A, b, x, lu=None, steps=3):
    """FP64 iterative refinement of an oracle solution with its own SuperLU
    factor (used where the raw oracle's residual is above the comparison
    tolerance)."""
    A = A.tocsc()
    if lu is None:
        lu = spl.splu(A)
    for _ in range(steps):
        x = x + lu.solve(b - A @ x)
    return x


def fields(omega, xlen, ylen, eps_tot, NPML, pol, L0, X, averaging=True):
    """Secondary fields from the primary field X (simulation.py:129-175).
    Returns (Ex, Ey, Hz) for Hz or (Hx, Hy, Ez) for Ez as (Nx, Ny) arrays."""
    eps_tot = np.asarray(eps_tot, dtype=np.float64)
    Nx, Ny = eps_tot.shape
    D = derivs(omega, xlen, ylen, Nx, Ny, NPML, L0)
    X = np.asarray(X).reshape(-1)
    if pol == 'Ez':
        MU0_ = MU_0 * L0
        hx = -1 / 1j / omega / MU0_ * D['Dyb'].dot(X)
        hy = 1 / 1j / omega / MU0_ * D['Dxb'].dot(X)
        return hx.reshape(Nx, Ny), hy.reshape(Nx, Ny), X.reshape(Nx, Ny)
    EPS0_ = EPSILON_0 * L0
    if averaging:
        vx = grid_average(EPS0_ * eps_tot, 'x').reshape(-1)
        vy = grid_average(EPS0_ * eps_tot, 'y').reshape(-1)
    else:
        vx = vy = (EPS0_ * eps_tot).reshape(-1)
    ex = 1 / 1j / omega * (sp.diags(1 / vy) @ D['Dyb']).dot(X)
    ey = -1 / 1j / omega * (sp.diags(1 / vx) @ D['Dxb']).dot(X)
    return ex.reshape(Nx, Ny), ey.reshape(Nx, Ny), X.reshape(Nx, Ny)


def flux_probe(pol, fields_dict, dl, direction_normal, center, width):
    """Poynting flux through a line (simulation.py:260-315)."""
    if direction_normal == 'x':
        ix = [center[0], center[0] + 1]
        iy = [int(center[1] - width / 2), int(center[1] + width / 2)]
    elif direction_normal == 'y':
        ix = [int(center[0] - width / 2), int(center[0] + width / 2)]
        iy = [center[1], center[1] + 1]
    else:
        raise ValueError("The value of direction_normal is neither x nor y!")
    if pol == 'Ez':
        Ez, Hx, Hy = fields_dict['Ez'], fields_dict['Hx'], fields_dict['Hy']
        blk = Ez[ix[0]:ix[1] + 1, iy[0]:iy[1] + 1]
        if direction_normal == 'x':
            Ex_ = grid_average(blk, 'x')[:-1, :-1]
            return dl * np.sum(-1 / 2 * np.real(Ex_ * np.conj(Hy[ix[0]:ix[1], iy[0]:iy[1]])))
        Ey_ = grid_average(blk, 'y')[:-1, :-1]
        return dl * np.sum(1 / 2 * np.real(Ey_ * np.conj(Hx[ix[0]:ix[1], iy[0]:iy[1]])))
    Hz, Ex, Ey = fields_dict['Hz'], fields_dict['Ex'], fields_dict['Ey']
    blk = Hz[ix[0]:ix[1] + 1, iy[0]:iy[1] + 1]
    if direction_normal == 'x':
        Hx_ = grid_average(blk, 'x')[:-1, :-1]
        return dl * np.sum(1 / 2 * np.real(Ey[ix[0]:ix[1], iy[0]:iy[1]] * np.conj(Hx_)))
    Hy_ = grid_average(blk, 'y')[:-1, :-1]
    return dl * np.sum(-1 / 2 * np.real(Ex[ix[0]:ix[1], iy[0]:iy[1]] * np.conj(Hy_)))


def p_scaling(omega, L0, Nx, Ny, NPML, xlen, ylen):
    """P = diag(sxf(i) syf(j)) with P A complex symmetric (both
    polarizations), so A^T = P A P^-1."""
    sxf = sfactor(xlen, L0, 'f', omega, Nx, NPML[0])
    syf = sfactor(ylen, L0, 'f', omega, Ny, NPML[1])
    return (sxf[:, None] * syf[None, :]).reshape(-1)


def adjoint_grad_eps_Ez(A, E, g, omega, L0):
    """Reference gradient dL/d(eps_r) for a real loss L of the complex field
    E = A^-1 b, given torch's grad_output g = dL/dconj(E) * 2:
    lambda = A^-T conj(g),  dL/deps = -omega^2 eps0 L0 Re(lambda * E).
    (dA/deps_p = omega^2 eps0' e_p e_p^T from linalg.py:53-54, 66.)"""
    lam = spl.spsolve(A.T.tocsc(), np.conj(g).reshape(-1))
    return -(omega ** 2) * (EPSILON_0 * L0) * np.real(lam * E.reshape(-1))


def adjoint_grad_eps_Hz(omega, xlen, ylen, eps_r, NPML, L0, E, g, averaging=True):
    """Reference gradient dL/d(eps_r) for Hz (derived from construct_A,
    linalg.py:69-93: A = Dxf' Tx^-1 Dxb' + Dyf' Ty^-1 Dyb' + omega^2 mu0' I
    with Tx, Ty the grid-averaged eps0' eps), by the chain rule through the
    edge permittivities with scipy's sparse derivative operators:
    lambda = A^-T conj(g), u = Dxf'^T lambda, v = Dxb' E,
    dL/d eps_x[q] = Re(u_q v_q) / eps_x[q]^2, spread onto eps_r by the
    averaging weights (1/2 on the cell and its -x neighbour)."""
    eps_r = np.asarray(eps_r, dtype=np.float64)
    Nx, Ny = eps_r.shape
    A = construct_A(omega, xlen, ylen, eps_r, NPML, 'Hz', L0, averaging=averaging)
    lam = spl.spsolve(A.T.tocsc(), np.conj(np.asarray(g)).reshape(-1))
    D = derivs(omega, xlen, ylen, Nx, Ny, NPML, L0)
    E = np.asarray(E).reshape(-1)
    e = EPSILON_0 * L0 * eps_r
    ex = grid_average(e, 'x') if averaging else e
    ey = grid_average(e, 'y') if averaging else e
    tx = (np.real((D['Dxf'].T @ lam) * (D['Dxb'] @ E)) / ex.reshape(-1) ** 2).reshape(Nx, Ny)
    ty = (np.real((D['Dyf'].T @ lam) * (D['Dyb'] @ E)) / ey.reshape(-1) ** 2).reshape(Nx, Ny)
    if averaging:
        grad = 0.5 * EPSILON_0 * L0 * (tx + np.roll(tx, -1, axis=0) + ty + np.roll(ty, -1, axis=1))
    else:
        grad = EPSILON_0 * L0 * (tx + ty)
    return grad.reshape(-1)


def kerr_adjoint_grad_Ez(omega, xlen, ylen, eps_r, NPML, L0, E, g, chi, region, eps_scale=False, eps_max=None):
    """Reference gradient dL/d(eps_r) at a converged Kerr solution E of
    (A + diag(w eps_nl(E))) E = b (w = omega^2 eps0 L0; newton_solve,
    nonlinear_solvers.py:57-115): the real 2n x 2n Newton Jacobian R of
    solver_complex2real (linalg.py:152-186) is transposed, R^T m = [Re g;
    Im g] is solved by SuperLU, mu = m_r + i m_i, and
    dL/d eps_p = -w Re(conj(mu_p) (1 + dnl_deps_p) E_p)."""
    eps_r = np.asarray(eps_r, dtype=np.float64)
    E = np.asarray(E).reshape(-1)
    n = E.size
    w = omega ** 2 * EPSILON_0 * L0
    A = construct_A(omega, xlen, ylen, eps_r, NPML, 'Ez', L0)
    eps_nl, dnl = kerr_terms(E, eps_r.reshape(-1), chi, np.asarray(region).reshape(-1), eps_scale, eps_max)
    dAde = dnl * w
    J11 = (A + sp.diags(w * eps_nl) + sp.diags(dAde * E)).tocsr()
    J12 = sp.diags(np.conj(dAde) * E).tocsr()
    R = sp.vstack((sp.hstack((J11.real + J12.real, -J11.imag + J12.imag)),
                   sp.hstack((J11.imag + J12.imag, J11.real - J12.real)))).tocsc()
    g = np.asarray(g).reshape(-1)
    m = spl.spsolve(R.T.tocsc(), np.concatenate([g.real, g.imag]))
    mu = m[:n] + 1j * m[n:]
    deps = 3 * chi * np.asarray(region).reshape(-1) * np.abs(E) ** 2 / (eps_max - 1) if eps_scale else 0.0
    return -w * np.real(np.conj(mu) * (1 + deps) * E)


# ---- mode source (fdfdpy/source/mode.py:62-108) ------------------------------
def mode_operator(pol, eps_slice, omega, dl, L0, average):
    """The 1-D periodic slice operator of insert_mode (mode.py:76-91):
    Ez: omega^2 mu0' T_eps + Dxf Dxb;  Hz: omega^2 mu0' T_eps + T_eps Dxf
    T_epsx^-1 Dxb, raw periodic differences of spacing dl.  `average`
    selects whether grid_average(eps, 'x') averages along the slice (a
    slice normal to y) or returns eps (normal to x: one row)."""
    e_sl = np.asarray(eps_slice, dtype=np.float64).reshape(-1)
    Ns = e_sl.size
    v = 1 / dl
    I = np.arange(Ns)
    Dxf = sp.csr_matrix((np.concatenate([-v * np.ones(Ns), v * np.ones(Ns)]),
                         (np.concatenate([I, I]), np.concatenate([I, (I + 1) % Ns]))), shape=(Ns, Ns))
    Dxb = sp.csr_matrix((np.concatenate([v * np.ones(Ns), -v * np.ones(Ns)]),
                         (np.concatenate([I, I]), np.concatenate([I, (I - 1) % Ns]))), shape=(Ns, Ns))
    EPS0_, MU0_ = EPSILON_0 * L0, MU_0 * L0
    T_eps = sp.diags(EPS0_ * e_sl)
    if pol == 'Ez':
        return (np.square(omega) * MU0_ * T_eps + Dxf.dot(Dxb)).tocsr()
    avg = (np.roll(e_sl, 1) + e_sl) / 2 if average else e_sl
    T_inv = sp.diags((EPS0_ * avg) ** (-1))
    return (np.square(omega) * MU0_ * T_eps + T_eps.dot(Dxf).dot(T_inv).dot(Dxb)).tocsr()


def mode_eigs(A1, order, sigma):
    """ARPACK shift-invert around sigma (linalg.py:110-119)."""
    return spl.eigs(A1, k=order, sigma=sigma, which='LM')


# ---- Kerr nonlinearity (fdfdpy/nonlinearity.py, nonlinear_solvers.py) ----------
def kerr_terms(E, eps_r, chi, region, eps_scale=False, eps_max=None):
    """eps_nl and dnl_de of one Kerr nonlinearity (nonlinearity.py:18-34);
    chi already divided by L0^2 (simulation.py:72)."""
    s = (eps_r - 1) / (eps_max - 1) if eps_scale else 1.0
    return 3 * chi * region * np.square(np.abs(E)) * s, 3 * chi * region * np.conj(E) * s


def solve_complex2real(A11, A12, b):
    """[Re A11 + Re A12, -Im A11 + Im A12; Im A11 + Im A12, Re A11 - Re A12]
    [xr; xi] = [br; bi] (linalg.py:152-186) by SuperLU."""
    b = np.asarray(b).astype(np.complex128).reshape(-1)
    n = b.size
    R = sp.vstack((sp.hstack((A11.real + A12.real, -A11.imag + A12.imag)),
                   sp.hstack((A11.imag + A12.imag, A11.real - A12.real)))).tocsc()
    x = spl.spsolve(R, np.concatenate([b.real, b.imag]))
    return x[:n] + 1j * x[n:]


def born_kerr_Ez(omega, xlen, ylen, eps_r, NPML, L0, src, chi, region, eps_scale=False, eps_max=None,
                 conv_threshold=1e-10, max_num_iter=50):
    """Born fixed point of born_solve (nonlinear_solvers.py:13-54) for one
    Kerr term, Ez, from the linear solution: E <- (A + Anl(E))^-1 b with
    Anl = diag(omega^2 eps0 L0 eps_nl) (simulation.py:57-68); returns
    (Ez, conv list), Ez being the last iteration's solve."""
    eps_r = np.asarray(eps_r, dtype=np.float64)
    A = construct_A(omega, xlen, ylen, eps_r, NPML, 'Ez', L0)
    b = (1j * omega * np.asarray(src)).reshape(-1).astype(np.complex128)
    E = solve(A, b)
    conv = []
    for _ in range(max_num_iter):
        eps_nl, _ = kerr_terms(E, eps_r.reshape(-1), chi, region.reshape(-1), eps_scale, eps_max)
        En = solve(A + sp.diags(omega ** 2 * EPSILON_0 * L0 * eps_nl), b)
        c = np.linalg.norm(En - E) / np.linalg.norm(En)
        conv.append(c)
        E = En
        if c < conv_threshold:
            break
    return E, conv


def newton_kerr_Ez(omega, xlen, ylen, eps_r, NPML, L0, src, chi, region, eps_scale=False, eps_max=None,
                   conv_threshold=1e-10, max_num_iter=50):
    """Newton iteration of newton_solve (nonlinear_solvers.py:57-115) for one
    Kerr term, Ez, from the linear solution; returns (Ez_nl, conv list)
    where Ez_nl is the final solve with the converged eps_nl."""
    eps_r = np.asarray(eps_r, dtype=np.float64)
    A = construct_A(omega, xlen, ylen, eps_r, NPML, 'Ez', L0)
    b = (1j * omega * np.asarray(src)).reshape(-1).astype(np.complex128)
    E = solve(A, b)
    n = E.size
    conv = []
    e0 = EPSILON_0 * L0
    for _ in range(max_num_iter):
        eps_nl, dnl = kerr_terms(E, eps_r.reshape(-1), chi, region.reshape(-1), eps_scale, eps_max)
        Anl = A + sp.diags(omega ** 2 * EPSILON_0 * L0 * eps_nl)
        f = Anl @ E - b
        dAde = dnl * omega ** 2 * e0
        J11 = Anl + sp.diags(dAde * E)
        J12 = sp.diags(np.conj(dAde) * E)
        En = E - solve_complex2real(J11.tocsr(), J12.tocsr(), f)
        c = np.linalg.norm(En - E) / np.linalg.norm(En)
        conv.append(c)
        E = En
        if c < conv_threshold:
            break
    eps_nl, _ = kerr_terms(E, eps_r.reshape(-1), chi, region.reshape(-1), eps_scale, eps_max)
    E_final = solve(A + sp.diags(omega ** 2 * EPSILON_0 * L0 * eps_nl), b)
    return E_final, conv
