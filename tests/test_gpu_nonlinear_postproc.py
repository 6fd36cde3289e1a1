"""Kerr kernel (K1-NL), factor reuse in the Kerr loops, the device flux
probe, the Hz adjoint gradient, the Kerr adjoint and the optimisation
wiring, each against the oracle (pinned to the reference's outputs, or to
finite differences where the reference has no counterpart)."""
import numpy as np
import pytest
import torch

from oracle import fdfd_oracle as O

pytestmark = pytest.mark.gpu
OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


def test_kerr_assemble_matches_nonlinearity_terms():
    """fdfd_kerr_assemble against nonlinearity.py:18-34 / compute_nl
    (oracle.kerr_terms), two nonlinearities accumulated, with and without
    eps scaling: relative 1e-14."""
    from fdfdpy_gb300 import Simulation
    from fdfdpy_gb300.nonlinear_solvers import KerrTerms
    rng = np.random.default_rng(6)
    Nx, Ny = 30, 26
    eps = 1 + 11 * rng.random((Nx, Ny))
    sim = Simulation(OMEGA, eps, 0.02, [4, 4], "Ez")
    r1 = (rng.random((Nx, Ny)) > 0.5).astype(float)
    r2 = rng.random((Nx, Ny))
    sim.add_nl(2.8e-18, r1)
    sim.add_nl(1.1e-18, r2, eps_scale=True, eps_max=12.0)
    E = (rng.standard_normal((Nx, Ny)) + 1j * rng.standard_normal((Nx, Ny))) * 1e3
    t = KerrTerms.of(sim)(E, eps_nl=True, jac=True, deps=True, de=True)
    w = OMEGA ** 2 * O.EPSILON_0 * 1e-6
    e1, d1 = O.kerr_terms(E.reshape(-1), eps.reshape(-1), 2.8e-18 / 1e-12, r1.reshape(-1))
    e2, d2 = O.kerr_terms(E.reshape(-1), eps.reshape(-1), 1.1e-18 / 1e-12, r2.reshape(-1), True, 12.0)
    want = {"eps_nl": e1 + e2, "dnl_de": d1 + d2, "jac_diag": (d1 + d2) * w * E.reshape(-1),
            "jac_off": np.conj((d1 + d2) * w) * E.reshape(-1),
            "dnl_deps": 3 * (1.1e-18 / 1e-12) * r2.reshape(-1) * np.abs(E.reshape(-1)) ** 2 / 11.0}
    for k, v in want.items():
        got = t[k].cpu().numpy()
        assert np.max(np.abs(got - v)) <= 1e-14 * np.max(np.abs(v)), k
    # the host attributes of compute_nl (simulation.py:57-68) come from the kernel too
    sim.compute_nl(E)
    assert np.max(np.abs(sim.eps_nl.reshape(-1) - want["eps_nl"])) <= 1e-14 * np.max(want["eps_nl"])


def test_newton_and_born_reuse_factors():
    """Factor reuse across Kerr iterations: fewer factorizations than
    iterations, same fields as the oracle's exact Newton (1e-9)."""
    from fdfdpy_gb300 import Simulation
    rng = np.random.default_rng(2)
    Nx, Ny, dl = 48, 40, 0.02
    eps = 1 + 11 * rng.random((Nx, Ny))
    region = np.zeros((Nx, Ny))
    region[16:32, 12:28] = 1
    sim = Simulation(OMEGA, eps, dl, [6, 6], "Ez")
    sim.src[10, 20] = 3e3
    sim.add_nl(2.8e-18, region)
    _, _, Ez, conv = sim.solve_fields_nl(solver_nl="newton", conv_threshold=1e-12)
    iters = int(np.count_nonzero(conv))
    assert sim.nl_stats["factorizations"] < iters, (sim.nl_stats, iters)
    Eo, _ = O.newton_kerr_Ez(OMEGA, Nx * dl, Ny * dl, eps, [6, 6], 1e-6, sim.src, 2.8e-18 / 1e-12, region,
                             conv_threshold=1e-12)
    assert np.linalg.norm(Ez.reshape(-1) - Eo) / np.linalg.norm(Eo) < 1e-9
    sim2 = Simulation(OMEGA, eps, dl, [6, 6], "Ez")
    sim2.src[10, 20] = 3e2
    sim2.add_nl(2.8e-18, region)
    _, _, Eb, cb = sim2.solve_fields_nl(solver_nl="born", conv_threshold=1e-12, max_num_iter=200)
    assert sim2.nl_stats["factorizations"] < int(np.count_nonzero(cb))
    Ebo, _ = O.born_kerr_Ez(OMEGA, Nx * dl, Ny * dl, eps, [6, 6], 1e-6, sim2.src, 2.8e-18 / 1e-12, region,
                            conv_threshold=1e-12, max_num_iter=200)
    assert np.linalg.norm(Eb.reshape(-1) - Ebo) / np.linalg.norm(Ebo) < 1e-8


@pytest.mark.parametrize("pol", ["Ez", "Hz"])
def test_flux_probe_device_matches_oracle(pol):
    from fdfdpy_gb300 import Simulation
    rng = np.random.default_rng(7)
    Nx, Ny, dl = 80, 70, 0.02
    eps = 1 + 3 * rng.random((Nx, Ny))
    sim = Simulation(OMEGA, eps, dl, [10, 10], pol)
    sim.src[40, 35] = 1
    sim.solve_fields()
    host = {k: v for k, v in sim.fields.items() if v is not None}
    for normal, center, width in (("x", [55, 35], 30), ("y", [40, 20], 41), ("x", [20, 30], 17)):
        got = sim.flux_probe(normal, center, width)
        want = O.flux_probe(pol, host, dl, normal, center, width)
        assert abs(got - want) <= 1e-12 * abs(want), (normal, got, want)
    # fields assigned by hand are uploaded and reduced on the device as well
    sim.fields = {k: (2 * v if v is not None else None) for k, v in sim.fields.items()}
    assert abs(sim.flux_probe("x", [55, 35], 30) - 4 * O.flux_probe(pol, host, dl, "x", [55, 35], 30)) <= \
        1e-12 * abs(4 * O.flux_probe(pol, host, dl, "x", [55, 35], 30))
    with pytest.raises(Exception):
        sim.flux_probe("x", [Nx - 1, 35], 10)        # the averaging neighbour leaves the grid


@pytest.mark.parametrize("averaging", [True, False])
def test_hz_adjoint_gradient_matches_oracle(averaging):
    from fdfdpy_gb300 import engine
    Nx, Ny, dl = 40, 36, 0.02
    rng = np.random.default_rng(8)
    eps = 1 + 11 * rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[8, 18] = 1
    k = 30 * Ny + 18
    op = engine.DeviceOperator(OMEGA, eps, Nx * dl, Ny * dl, [6, 6], "Hz", 1e-6, averaging=averaging)
    fac = engine.Factor(engine.symbolic_for(Nx, Ny), "c128").numeric(op)
    b = engine.as_c128(1j * OMEGA * src).reshape(-1)
    E = fac.solve(b)
    g = torch.zeros_like(E)
    g[k] = 2 * E[k]
    lam = fac.solve(torch.conj(g), transpose=True)
    grad = op.grad_eps(lam, E).cpu().numpy()
    ref = O.adjoint_grad_eps_Hz(OMEGA, Nx * dl, Ny * dl, eps, [6, 6], 1e-6, E.cpu().numpy(), g.cpu().numpy(),
                                averaging=averaging)
    assert np.linalg.norm(grad - ref) <= 1e-9 * np.linalg.norm(ref)


def test_autograd_solve_hz_matches_finite_differences():
    from fdfdpy_gb300.adjoint import solve
    Nx, Ny, dl = 40, 36, 0.02
    rng = np.random.default_rng(9)
    eps = 1 + 11 * rng.random((Nx, Ny))
    src = np.zeros((Nx, Ny))
    src[8, 18] = 1
    s = torch.tensor(src, device="cuda")

    def J_of(e):
        return float(solve(torch.tensor(e, device="cuda"), s, OMEGA, dl, [6, 6], "Hz")[30, 18].abs() ** 2)
    e = torch.tensor(eps, device="cuda", requires_grad=True)
    (solve(e, s, OMEGA, dl, [6, 6], "Hz")[30, 18].abs() ** 2).backward()
    g = e.grad.cpu().numpy().reshape(-1)
    pix = rng.choice(Nx * Ny, 16, replace=False)
    fd = []
    for p in pix:
        ep, em = eps.copy(), eps.copy()
        ep.flat[p] += 1e-5
        em.flat[p] -= 1e-5
        fd.append((J_of(ep) - J_of(em)) / 2e-5)
    fd = np.array(fd)
    assert np.linalg.norm(g[pix] - fd) <= 1e-6 * np.linalg.norm(fd)


@pytest.mark.parametrize("scale", [False, True])
def test_kerr_adjoint_matches_oracle_gradient(scale):
    """The adjoint of the Newton Jacobian at the converged Kerr field
    (spec: the Kerr Jacobian differentiated like the linear solve)
    against the oracle's real 2n x 2n transposed solve (itself pinned to
    finite differences on the CPU): 1e-8 relative."""
    from fdfdpy_gb300.adjoint import solve_kerr_ez
    rng = np.random.default_rng(5)
    Nx, Ny, dl, chi = 24, 20, 0.02, 2.8e-18
    eps = 1 + 11 * rng.random((Nx, Ny))
    region = np.zeros((Nx, Ny))
    region[8:16, 6:14] = 1
    src = np.zeros((Nx, Ny))
    src[5, 10] = 2e3
    emax = 12.0 if scale else None
    k = (18, 10)
    e = torch.tensor(eps, device="cuda", requires_grad=True)
    E = solve_kerr_ez(e, torch.tensor(src, device="cuda"), OMEGA, dl, [4, 4], chi, region, scale, emax)
    (E[k].abs() ** 2).backward()
    g = e.grad.cpu().numpy().reshape(-1)
    Eo, conv = O.newton_kerr_Ez(OMEGA, Nx * dl, Ny * dl, eps, [4, 4], 1e-6, src, chi / 1e-12, region, scale, emax,
                                conv_threshold=1e-14, max_num_iter=60)
    assert np.linalg.norm(E.detach().cpu().numpy().reshape(-1) - Eo) <= 1e-9 * np.linalg.norm(Eo)
    go = np.zeros(Nx * Ny, complex)
    go[k[0] * Ny + k[1]] = 2 * Eo[k[0] * Ny + k[1]]
    ref = O.kerr_adjoint_grad_Ez(OMEGA, Nx * dl, Ny * dl, eps, [4, 4], 1e-6, Eo, go, chi / 1e-12, region, scale,
                                 emax)
    assert np.linalg.norm(g - ref) <= 1e-8 * np.linalg.norm(ref)


def test_design_region_optimisation_step_increases_objective():
    """init_design_region (simulation.py:344-369) + the differentiable
    Simulation solve: the projected gradient steps of adjoint.design_step
    raise |Ez|^2 at a probe, and the Simulation-level gradient equals the
    oracle's float64 gradient over the design region."""
    from fdfdpy_gb300 import Simulation
    from fdfdpy_gb300.adjoint import design_step
    N, dl = 60, 0.02
    eps = np.ones((N, N))
    region = np.zeros((N, N))
    region[20:40, 20:40] = 1
    sim = Simulation(OMEGA, eps, dl, [10, 10], "Ez")
    sim.src[12, 30] = 1
    np.random.seed(0)
    sim.init_design_region(region, 6.0, style='random')
    probe = (48, 30)

    def objective(fields):
        return fields[2][probe].abs() ** 2
    J0, g = design_step(sim, region, objective, 6.0, step=0.0)     # gradient only
    A = O.construct_A(OMEGA, N * dl, N * dl, sim.eps_r, [10, 10], "Ez", 1e-6)
    Eo = O.solve(A, 1j * OMEGA * sim.src.reshape(-1))
    go = np.zeros(N * N, complex)
    go[probe[0] * N + probe[1]] = 2 * Eo[probe[0] * N + probe[1]]
    ref = O.adjoint_grad_eps_Ez(A, Eo, go, OMEGA, 1e-6) * region.reshape(-1)
    assert np.linalg.norm(g.cpu().numpy().reshape(-1) - ref) <= 1e-9 * np.linalg.norm(ref)
    Js = [J0]
    for _ in range(3):
        Jk, _ = design_step(sim, region, objective, 6.0, step=0.2)
        Js.append(Jk)
    assert Js[-1] > Js[0], Js
    assert sim.eps_r[region == 0].max() == 1.0 and 1.0 <= sim.eps_r.min() and sim.eps_r.max() <= 6.0


def test_init_design_region_matches_reference():
    """init_design_region for every style against the reference's own
    outputs (tests/golden/design.npz; numpy's RNG seeded alike)."""
    from pathlib import Path
    from fdfdpy_gb300 import Simulation
    g = np.load(Path(__file__).resolve().parent / "golden" / "design.npz")
    for style in ("full", "halfway", "empty", "random", "other"):
        eps = g["eps"].copy()
        sim = Simulation(OMEGA, eps, 0.02, [3, 3], "Ez")
        np.random.seed(5)
        sim.init_design_region(g["region"], 7.5, style=style)
        assert np.array_equal(sim.eps_r, g[style]), style
        if style == "halfway":
            assert sim.eps_r is eps                 # modified in place, as the reference does
