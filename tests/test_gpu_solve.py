"""GPU multifrontal factor + solve against the oracle (SuperLU) and the
golden fields of the reference.

Bars (fields, relative 2-norm): complex128 factor <= 1e-10; complex64
factor + FP64 refinement to a residual of 1e-10 <= 1e-8 (field error is
bounded by cond(A) x residual; the refined residual itself is checked
<= 1e-10).
"""
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import fdfd_oracle as O

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


@pytest.fixture(scope="module")
def eng():
    from fdfdpy_gb300 import engine
    engine.device()
    return engine


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _problem(Nx, Ny, pol, seed=0, npml=(6, 5), dl=0.02):
    rng = np.random.default_rng(seed)
    eps = 1 + 11 * rng.random((Nx, Ny))
    A = O.construct_A(OMEGA, Nx * dl, Ny * dl, eps, list(npml), pol, 1e-6)
    return eps, A, rng


@pytest.mark.parametrize("Nx,Ny,pol,leaf", [(3, 3, "Ez", 1), (8, 8, "Ez", 4), (17, 13, "Hz", 16),
                                            (64, 48, "Ez", 64), (97, 131, "Hz", 64), (150, 7, "Ez", 16)])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_solve_matches_superlu(eng, Nx, Ny, pol, leaf, prec):
    npml = (min(6, Nx // 3), min(5, Ny // 3))
    eps, A, rng = _problem(Nx, Ny, pol, npml=npml)
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, list(npml), pol, 1e-6)
    fac = eng.Factor(eng.Symbolic(Nx, Ny, leaf), prec, max_nrhs=3).numeric(op)
    b = rng.standard_normal((3, Nx * Ny)) + 1j * rng.standard_normal((3, Nx * Ny))
    x = fac.solve(b, tol=1e-12 if prec == "c128" else 1e-10, max_iter=40, raise_on_fail=True)
    x = x.cpu().numpy()
    st = fac.stats()
    assert st["rel_residual"] <= (1e-12 if prec == "c128" else 1e-10)
    for k in range(3):
        xr = O.solve(A, b[k])
        assert rel(x[k], xr) < (1e-10 if prec == "c128" else 1e-8), (k, st)
        assert np.linalg.norm(A @ x[k] - b[k]) / np.linalg.norm(b[k]) < 1e-10


def test_single_application_and_transpose(eng):
    Nx, Ny = 40, 36
    eps, A, rng = _problem(Nx, Ny, "Ez", seed=2)
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [6, 5], "Ez", 1e-6)
    fac = eng.Factor(eng.Symbolic(Nx, Ny), "c128").numeric(op)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    x1 = fac.apply_inverse(b).cpu().numpy()
    assert rel(x1, O.solve(A, b)) < 1e-10
    xt = fac.apply_inverse(b, transpose=True).cpu().numpy()
    assert rel(xt, O.solve(A.T.tocsr(), b)) < 1e-10
    xt2 = fac.solve(b, transpose=True, tol=1e-13, max_iter=5).cpu().numpy()
    assert np.linalg.norm(A.T @ xt2 - b) / np.linalg.norm(b) < 1e-12


def test_factor_is_deterministic(eng):
    Nx, Ny = 70, 70
    eps, A, rng = _problem(Nx, Ny, "Hz", seed=4)
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [6, 5], "Hz", 1e-6)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    sym = eng.Symbolic(Nx, Ny)
    xs = []
    for _ in range(2):
        fac = eng.Factor(sym, "c64").numeric(op)
        xs.append(fac.apply_inverse(b).cpu().numpy())
    assert np.array_equal(xs[0], xs[1])


def test_ez200_matches_reference_fields(eng):
    from fdfdpy_gb300 import Simulation
    g = np.load(GOLD / "ez200.npz")
    N = 200
    eps = np.ones((N, N))
    eps[80:120, 80:120] = 12
    for prec, tol in (("c128", 1e-10), ("c64", 1e-8)):
        sim = Simulation(OMEGA, eps, 0.02, [15, 15], "Ez")
        sim.src[100, 100] = 1
        Hx, Hy, Ez = sim.solve_fields(precision=prec)
        s = g["sample"]
        for got, key in ((Hx, "Hx"), (Hy, "Hy"), (Ez, "Ez")):
            assert rel(got.reshape(-1)[s], g[key]) < tol, (prec, key)
        norms = [np.linalg.norm(Hx), np.linalg.norm(Hy), np.linalg.norm(Ez)]
        assert np.allclose(norms, g["norms"], rtol=tol)
        assert sim.last_solve_stats["rel_residual"] <= (1e-12 if prec == "c128" else 1e-10)


def test_hz_blocks_matches_reference_fields(eng):
    from fdfdpy_gb300 import Simulation
    g = np.load(GOLD / "hz128_blocks.npz")
    sim = Simulation(OMEGA, g["eps"], 0.01, [20, 20], "Hz")
    sim.src[30, :] = 1
    for prec, tol in (("c128", 1e-10), ("c64", 1e-8)):
        Ex, Ey, Hz = sim.solve_fields(precision=prec)
        assert rel(Hz, g["Hz"]) < tol and rel(Ex, g["Ex"]) < tol and rel(Ey, g["Ey"]) < tol


def test_zero_source_and_factor_reuse(eng):
    from fdfdpy_gb300 import Simulation
    eps = np.ones((30, 30))
    sim = Simulation(OMEGA, eps, 0.02, [5, 5], "Ez")
    Hx, Hy, Ez = sim.solve_fields()
    assert Ez.dtype == np.float64 and not Ez.any() and not Hx.any()
    sim.src[15, 15] = 1
    sim.solve_fields()
    fac = next(iter(sim._factors.values()))
    sim.src[10, 12] = 2
    sim.solve_fields()
    assert next(iter(sim._factors.values())) is fac  # only the source changed
    sim.eps_r = eps * 2
    assert sim.fields["Ez"] is None and not sim._factors


def test_not_converged_is_reported(eng):
    from fdfdpy_gb300 import _native as N
    Nx, Ny = 60, 60
    eps, A, rng = _problem(Nx, Ny, "Ez", seed=9)
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [6, 5], "Ez", 1e-6)
    fac = eng.Factor(eng.Symbolic(Nx, Ny), "c64").numeric(op)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    with pytest.raises(N.NotConverged):
        fac.solve(b, tol=1e-15, max_iter=0, raise_on_fail=True)


@pytest.mark.parametrize("prec", ["c64", "c64tc", "c128"])
def test_gmres_refinement_matches_superlu(eng, prec):
    Nx, Ny = 230, 170
    eps, A, rng = _problem(Nx, Ny, "Hz", seed=12, npml=(12, 12))
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [12, 12], "Hz", 1e-6)
    fac = eng.Factor(eng.symbolic_for(Nx, Ny), prec, max_nrhs=2).numeric(op)
    b = rng.standard_normal((2, Nx * Ny)) + 1j * rng.standard_normal((2, Nx * Ny))
    x = fac.solve(b, tol=1e-11, max_iter=40, method="gmres", raise_on_fail=True).cpu().numpy()
    assert fac.stats()["rel_residual"] <= 1e-11
    for k in range(2):
        assert np.linalg.norm(A @ x[k] - b[k]) / np.linalg.norm(b[k]) < 1e-11
        assert rel(x[k], O.solve(A, b[k])) < 1e-8
    xt = fac.solve(b[0], transpose=True, tol=1e-11, max_iter=40, method="gmres", raise_on_fail=True).cpu().numpy()
    assert np.linalg.norm(A.T @ xt - b[0]) / np.linalg.norm(b[0]) < 1e-11


@pytest.mark.parametrize("prec", ["c128", "c64"])
@pytest.mark.parametrize("leaf", [16, 64])
def test_whole_front_and_panel_kernels_agree(eng, prec, leaf):
    """Small fronts factored in one launch per level (the whole front in
    shared memory) and the same fronts through the per-panel kernels give
    the same solution, and both match SuperLU."""
    Nx, Ny = 150, 122
    eps, A, rng = _problem(Nx, Ny, "Hz", seed=21, npml=(10, 10))
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [10, 10], "Hz", 1e-6)
    sym = eng.Symbolic(Nx, Ny, leaf)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    xr = O.solve(A, b)
    xs = []
    for limit in (-1, 0, 100000):  # default, never, as large as shared memory allows
        fac = eng.Factor(sym, prec, fused_max_m=limit).numeric(op)
        x0 = fac.apply_inverse(b).cpu().numpy()  # one application, no refinement
        if prec == "c128":
            assert rel(x0, xr) < 1e-10, limit
        else:
            assert rel(x0, xr) < 1e-2, limit
        x = fac.solve(b, tol=1e-12 if prec == "c128" else 1e-10, max_iter=40, raise_on_fail=True)
        xs.append(x.cpu().numpy())
        assert rel(xs[-1], xr) < (1e-10 if prec == "c128" else 1e-8), limit
    for x in xs[1:]:
        assert rel(xs[0], x) < (1e-10 if prec == "c128" else 1e-8)


def test_static_pivot_lifts_are_counted_on_both_paths(eng):
    Nx, Ny = 90, 90
    eps, A, rng = _problem(Nx, Ny, "Ez", seed=22)
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [6, 5], "Ez", 1e-6)
    sym = eng.Symbolic(Nx, Ny, 64)
    counts = []
    for limit in (-1, 0):
        fac = eng.Factor(sym, "c128", pivot_tol=0.3, fused_max_m=limit).numeric(op)
        counts.append(fac.stats()["tiny_pivots"])
    assert counts[0] > 0 and counts[1] > 0
    # same pivots up to rounding: only values at the threshold may differ
    assert abs(counts[0] - counts[1]) <= max(2, counts[0] // 10)


@pytest.mark.parametrize("prec,nrhs", [("c128", 1), ("c128", 3), ("c64", 2)])
def test_cooperative_levels_solve(eng, prec, nrhs):
    """A grid large enough that the top levels (separators of >= 256
    unknowns) run the pipelined cooperative substitutions, forward and
    transposed, checked by the residual of the operator (scipy CSR)."""
    Nx, Ny = 700, 520
    eps, A, rng = _problem(Nx, Ny, "Hz", seed=31, npml=(15, 15))
    op = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [15, 15], "Hz", 1e-6)
    fac = eng.Factor(eng.symbolic_for(Nx, Ny), prec, max_nrhs=nrhs).numeric(op)
    b = rng.standard_normal((nrhs, Nx * Ny)) + 1j * rng.standard_normal((nrhs, Nx * Ny))
    tol = 1e-9 if prec == "c128" else 1e-2  # one application of the complex64 factor
    for transpose in (False, True):
        x = fac.apply_inverse(b, transpose=transpose).cpu().numpy().reshape(nrhs, -1)
        M = A.T.tocsr() if transpose else A
        for k in range(nrhs):
            assert np.linalg.norm(M @ x[k] - b[k]) / np.linalg.norm(b[k]) < tol, (transpose, k)
    x = fac.solve(b, tol=1e-11, max_iter=30, raise_on_fail=True).cpu().numpy().reshape(nrhs, -1)
    for k in range(nrhs):
        assert np.linalg.norm(A @ x[k] - b[k]) / np.linalg.norm(b[k]) < 1e-11


def test_refinement_against_another_operator(eng):
    """The factor of one operator preconditions the refinement for a nearby
    operator: the residual is taken with the operator passed to the solve
    (applied matrix-free), not the stored coefficients of the factored one."""
    Nx, Ny = 90, 80
    eps, A, rng = _problem(Nx, Ny, "Hz", seed=41)
    eps2 = eps * 1.002
    A2 = O.construct_A(OMEGA, Nx * 0.02, Ny * 0.02, eps2, [6, 5], "Hz", 1e-6)
    op1 = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [6, 5], "Hz", 1e-6)
    op2 = eng.DeviceOperator(OMEGA, eps2, Nx * 0.02, Ny * 0.02, [6, 5], "Hz", 1e-6)
    fac = eng.Factor(eng.Symbolic(Nx, Ny), "c128").numeric(op1)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    x1 = fac.solve(b, tol=1e-12, max_iter=5, raise_on_fail=True).cpu().numpy()
    assert np.linalg.norm(A @ x1 - b) / np.linalg.norm(b) < 1e-12
    x2 = fac.solve(b, tol=1e-12, max_iter=60, op=op2, raise_on_fail=True).cpu().numpy()
    assert np.linalg.norm(A2 @ x2 - b) / np.linalg.norm(b) < 1e-12
    assert fac.stats()["refine_iters"] > 1


def test_released_factor_memory_is_reused(eng):
    """A factor of the shared symbolic analysis that is released keeps its
    device memory for the next factor of the same grid and precision; the
    reused factor is refactored from scratch (a different operator solves
    to its own solution)."""
    Nx, Ny = 66, 58
    eps, A, rng = _problem(Nx, Ny, "Ez", seed=51)
    eps2 = eps[::-1].copy()
    A2 = O.construct_A(OMEGA, Nx * 0.02, Ny * 0.02, eps2, [6, 5], "Ez", 1e-6)
    op1 = eng.DeviceOperator(OMEGA, eps, Nx * 0.02, Ny * 0.02, [6, 5], "Ez", 1e-6)
    op2 = eng.DeviceOperator(OMEGA, eps2, Nx * 0.02, Ny * 0.02, [6, 5], "Ez", 1e-6)
    sym = eng.symbolic_for(Nx, Ny)
    b = rng.standard_normal(Nx * Ny) + 1j * rng.standard_normal(Nx * Ny)
    f1 = eng.Factor(sym, "c128").numeric(op1)
    h1 = f1.handle.value
    assert rel(f1.apply_inverse(b).cpu().numpy(), O.solve(A, b)) < 1e-10
    del f1
    f2 = eng.Factor(sym, "c128", pivot_tol=0.3).numeric(op2)
    assert f2.handle.value == h1
    assert f2.stats()["tiny_pivots"] > 0  # the new factor's own settings apply
    f2 = None
    f3 = eng.Factor(sym, "c128").numeric(op2)
    assert f3.handle.value == h1 and f3.stats()["tiny_pivots"] == 0
    assert rel(f3.apply_inverse(b).cpu().numpy(), O.solve(A2, b)) < 1e-10
    other = eng.Factor(eng.Symbolic(Nx, Ny), "c128")  # a private analysis never takes a parked factor
    assert other.handle.value != h1


@pytest.mark.parametrize("pol", ["Ez", "Hz"])
def test_solver_direct_general_csr(eng, pol):
    """solver_direct on a scipy matrix that did not come from construct_A
    (the reference accepts any sparse A, linalg.py:122-149): A + a random
    diagonal (the A + Anl of simulation.py:125), assembled on the host by
    the oracle, is factored from its five diagonals; other patterns raise."""
    import scipy.sparse as sp
    from fdfdpy_gb300.linalg import solver_direct
    eps, A, rng = _problem(40, 33, pol, seed=3)
    A2 = (A + sp.diags(1e11 * rng.random(A.shape[0]))).tocsr()
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    for prec, tol in (("c128", 1e-10), ("c64", 1e-8)):
        x = solver_direct(A2, b, precision=prec)
        assert rel(x, O.solve(A2, b)) < tol, prec
    with pytest.raises(ValueError):
        solver_direct(sp.random(A.shape[0], A.shape[0], 0.01, format="csr") + sp.eye(A.shape[0]), b)


@pytest.mark.parametrize("prec", ["c64tc", "c128"])
def test_graph_replay_matches_direct_launches(eng, prec):
    """The factorization captured as a CUDA graph at the first call and
    replayed afterwards (with a new operator each time, whose coefficients
    are evaluated outside the graph) gives bitwise the same factor as direct
    launches; the tensor-core form's look-ahead stream is part of the graph."""
    N = 300 if prec == "c64tc" else 120
    rng = np.random.default_rng(21)
    sym = eng.symbolic_for(N, N)
    b = eng.as_c128(rng.standard_normal(N * N) + 1j * rng.standard_normal(N * N))
    g = eng.Factor(sym, prec)
    d = eng.Factor(sym, prec)
    d.set_graphs(False)
    for seed in range(3):
        eps = 1 + 11 * np.random.default_rng(seed).random((N, N))
        op = eng.DeviceOperator(OMEGA, eps, N * 0.02, N * 0.02, [10, 10], "Hz", 1e-6)
        xg = g.numeric(op).apply_inverse(b).cpu().numpy()
        xd = d.numeric(op).apply_inverse(b).cpu().numpy()
        assert np.array_equal(xg, xd), seed
