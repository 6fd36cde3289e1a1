"""The oracle's reference gradients (no counterpart in the reference, which
has no derivative with respect to eps) against central finite differences
of the oracle's own solves: Hz (edge-averaged and plain permittivities) and
the Kerr-nonlinear Ez solve at its Newton fixed point.  These pin the CPU
gradients the GPU adjoint tests compare against."""
import numpy as np

from oracle import fdfd_oracle as O

OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


def _fd(fun, eps, pixels, h):
    out = []
    for p in pixels:
        ep, em = eps.copy(), eps.copy()
        ep.flat[p] += h
        em.flat[p] -= h
        out.append((fun(ep) - fun(em)) / (2 * h))
    return np.array(out)


def test_hz_gradient_matches_finite_differences():
    rng = np.random.default_rng(4)
    Nx, Ny, dl = 22, 18, 0.02
    eps = 1 + 11 * rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[5, 9] = 1
    b = 1j * OMEGA * src.reshape(-1)
    k = 16 * Ny + 9
    for averaging in (True, False):
        def J(e):
            A = O.construct_A(OMEGA, Nx * dl, Ny * dl, e, [4, 4], "Hz", 1e-6, averaging=averaging)
            return abs(O.solve(A, b)[k]) ** 2
        A = O.construct_A(OMEGA, Nx * dl, Ny * dl, eps, [4, 4], "Hz", 1e-6, averaging=averaging)
        E = O.solve(A, b)
        g = np.zeros(Nx * Ny, complex)
        g[k] = 2 * E[k]
        grad = O.adjoint_grad_eps_Hz(OMEGA, Nx * dl, Ny * dl, eps, [4, 4], 1e-6, E, g, averaging=averaging)
        pix = rng.choice(Nx * Ny, 12, replace=False)
        fd = _fd(J, eps, pix, 1e-5)
        assert np.linalg.norm(grad[pix] - fd) <= 1e-6 * np.linalg.norm(fd), averaging


def test_kerr_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    Nx, Ny, dl, chi = 24, 20, 0.02, 2.8e-18 / 1e-12
    eps = 1 + 11 * rng.random((Nx, Ny))
    region = np.zeros((Nx, Ny))
    region[8:16, 6:14] = 1
    src = np.zeros((Nx, Ny))
    src[5, 10] = 2e3
    k = 18 * Ny + 10
    for scale in (False, True):
        emax = 12.0 if scale else None

        def J(e):
            E, conv = O.newton_kerr_Ez(OMEGA, Nx * dl, Ny * dl, e, [4, 4], 1e-6, src, chi, region, scale, emax,
                                       conv_threshold=1e-14, max_num_iter=60)
            return abs(E[k]) ** 2
        E, conv = O.newton_kerr_Ez(OMEGA, Nx * dl, Ny * dl, eps, [4, 4], 1e-6, src, chi, region, scale, emax,
                                   conv_threshold=1e-14, max_num_iter=60)
        assert conv[0] > 1e-6                   # genuinely nonlinear
        g = np.zeros(Nx * Ny, complex)
        g[k] = 2 * E[k]
        grad = O.kerr_adjoint_grad_Ez(OMEGA, Nx * dl, Ny * dl, eps, [4, 4], 1e-6, E, g, chi, region, scale, emax)
        pix = np.concatenate([rng.choice(np.flatnonzero(region.reshape(-1)), 6, replace=False),
                              rng.choice(np.flatnonzero(region.reshape(-1) == 0), 6, replace=False)])
        fd = _fd(J, eps, pix, 1e-5)
        assert np.linalg.norm(grad[pix] - fd) <= 1e-5 * np.linalg.norm(fd), scale
