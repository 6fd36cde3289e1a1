"""Kerr nonlinear solves on the GPU (born_solve / newton_solve) against the
oracle's restatement of the reference's Newton iteration (real 2n x 2n
solves with SuperLU), and Born == Newton (the reference's
test_nonlinear_solvers check, here on the nonlinear fields)."""
import numpy as np
import pytest

from oracle import fdfd_oracle as O

pytestmark = pytest.mark.gpu


def _waveguide(dl=0.02):
    n0, omega, chi3 = 3.4, 2 * np.pi * 200e12, 2.8e-18
    wv = int(1 / dl)
    Nx, Ny = int(5 / dl), int(3.5 / dl)
    eps = np.ones((Nx, Ny))
    eps[:, int(Ny / 2 - wv / 2):int(Ny / 2 + wv / 2)] = n0 ** 2
    region = np.zeros_like(eps)
    Lv = int(4 / dl)
    region[int(Nx / 2 - Lv / 2):int(Nx / 2 + Lv / 2), int(Ny / 2 - wv / 2):int(Ny / 2 + wv / 2)] = 1
    return n0, omega, chi3, eps, region, wv


def test_newton_matches_oracle_small():
    from fdfdpy_gb300 import Simulation
    rng = np.random.default_rng(2)
    Nx, Ny, dl = 48, 40, 0.02
    omega = 2 * np.pi * O.C_0 / 1.55e-6
    eps = 1 + 11 * rng.random((Nx, Ny))
    region = np.zeros((Nx, Ny))
    region[16:32, 12:28] = 1
    sim = Simulation(omega, eps, dl, [6, 6], "Ez")
    sim.src[10, 20] = 3e3  # eps_nl reaches ~10: strongly nonlinear, Newton converges
    chi = 2.8e-18
    sim.add_nl(chi, region)
    Hx, Hy, Ez, conv = sim.solve_fields_nl(solver_nl="newton", conv_threshold=1e-12)
    Eo, conv_o = O.newton_kerr_Ez(omega, Nx * dl, Ny * dl, eps, [6, 6], 1e-6, sim.src, chi / 1e-12, region,
                                  conv_threshold=1e-12)
    assert conv_o[-1] < 1e-12 and len(conv_o) > 1 and conv_o[0] > 1e-8  # genuinely nonlinear
    assert np.linalg.norm(Ez.reshape(-1) - Eo) / np.linalg.norm(Eo) < 1e-9
    assert sim.fields_nl["Ez"] is Ez


def test_born_equals_newton_waveguide():
    from fdfdpy_gb300 import Simulation
    n0, omega, chi3, eps, region, wv = _waveguide(dl=0.02)
    Nx, Ny = eps.shape
    sim = Simulation(omega, eps, 0.02, [15, 15], "Ez")
    sim.add_mode(n0, "x", [17, int(Ny / 2)], wv * 3)
    sim.setup_modes()
    sim.add_nl(chi3, region, eps_scale=True, eps_max=np.max(eps))
    for srcval in np.logspace(1, 3, 3):
        sim.setup_modes()
        sim.src *= srcval
        _, _, En, cn = sim.solve_fields_nl(solver_nl="newton")
        _, _, Eb, cb = sim.solve_fields_nl(solver_nl="born")
        assert np.linalg.norm(En - Eb) / np.linalg.norm(Eb) < 1e-7
