"""Generate golden vectors by running the reference fdfdpy itself.

Run where a checkout of the reference is available, naming it with
``--reference PATH`` (or the environment variable FDFDPY_REFERENCE):

    python tests/golden/make_golden.py --reference PATH [--only kerr|hz2048]

The reference imports pyMKL (absent here) and matplotlib (absent); both are
replaced by sys.modules shims before import:
  * pyMKL.pardisoSolver -> an exact SuperLU factor (scipy splu), so the
    reference's default solver='pardiso' path runs through SuperLU;
  * matplotlib          -> an empty module (plotting is not exercised).
The reference's Hz branch calls an unimported ``eye`` (fdfdpy/linalg.py:93);
the shim sets ``fdfdpy.linalg.eye = scipy.sparse.eye`` (its evident intent).

Outputs (small .npz files beside this script) hold inputs and outputs of
sfactor/construct_A/derivs/solve_fields/mode sources and of the Kerr
solvers (solve_fields_nl, Newton and Born) at sizes that take seconds.
Nothing at test time reads the reference.  `--only kerr` writes only the
Kerr fixture; `--only hz2048` writes the sampled fixture of the 2048 x 2048
Hz solve (about 15 minutes and 40 GB of host memory: the reference's
default solver path through the exact-LU shim, then FP64 iterative
refinement with the same factor); `--only kerr_sweep` the Kerr Newton
amplitude sweep at 128 x 128 (a few minutes); `--only design` the outputs
of init_design_region.
"""
from __future__ import annotations

import os
import sys
import types
from pathlib import Path

# SuperLU is single-threaded; a multi-threaded BLAS under it only spins on
# its small dense calls (measured: 107 s against 0.33 s for one 128^2 solve)
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
os.environ.setdefault("OMP_NUM_THREADS", "1")

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

OUT = Path(__file__).resolve().parent
REF = os.environ.get("FDFDPY_REFERENCE")


LAST_FACTOR = []   # the shim's most recent factor (kept for refinement)


def install_shims():
    if not REF or not Path(REF, "fdfdpy").is_dir():
        raise SystemExit("name the reference checkout: --reference PATH (or FDFDPY_REFERENCE)")
    pm = types.ModuleType("pyMKL")

    class pardisoSolver:  # exact LU stand-in for MKL PARDISO
        def __init__(self, A, mtype):
            self.A = sp.csc_matrix(A)

        def factor(self):
            self.lu = spl.splu(self.A)
            LAST_FACTOR[:] = [self.A, self.lu]

        def solve(self, b):
            return self.lu.solve(np.asarray(b))

        def clear(self):
            pass

    pm.pardisoSolver = pardisoSolver
    sys.modules["pyMKL"] = pm
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    mpl.pylab = mpl.pyplot
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = mpl.pyplot
    sys.modules["matplotlib.pylab"] = mpl.pyplot
    sys.path.insert(0, REF)
    import fdfdpy.linalg as L
    L.eye = sp.eye


def canon(A):
    A = sp.csr_matrix(A, copy=True)
    A.sort_indices()
    return A


def main():
    install_shims()
    import warnings
    warnings.simplefilter("ignore")
    from fdfdpy import Simulation
    from fdfdpy.constants import C_0
    from fdfdpy.linalg import construct_A
    from fdfdpy.pml import create_sfactor

    omega155 = 2 * np.pi * C_0 / 1.55e-6

    # 1. stretch factors
    sf = {}
    for tag, (wlen, Nw, npml, om, L0) in {
        "a": (4.0, 200, 15, omega155, 1e-6),
        "b": (20.48, 2048, 20, omega155, 1e-6),
        "c": (3.4, 17, 4, 2 * np.pi * 200e12, 1e-6),
        "d": (0.05, 50, 10, 100.0, 1e-4),
        "e": (1.0, 10, 0, omega155, 1e-6),
    }.items():
        sf[f"{tag}_args"] = np.array([wlen, Nw, npml, om, L0])
        sf[f"{tag}_f"] = create_sfactor([0, wlen], L0, "f", om, Nw, npml)
        sf[f"{tag}_b"] = create_sfactor([0, wlen], L0, "b", om, Nw, npml)
    np.savez_compressed(OUT / "sfactors.npz", **sf)

    # 2. small operators, derivatives and solved fields (all three solvers
    #    paths agree: scipy spsolve and the pardiso stand-in)
    rng = np.random.default_rng(1234)
    cases = {
        "ez_24x17": (24, 17, [5, 4], "Ez", 0.02, omega155, 1e-6),
        "hz_24x17": (24, 17, [5, 4], "Hz", 0.02, omega155, 1e-6),
        "ez_40x40": (40, 40, [10, 10], "Ez", 0.02, omega155, 1e-6),
        "hz_33x20_npml0": (33, 20, [0, 3], "Hz", 0.05, 2 * np.pi * 200e12, 1e-6),
        "ez_12x9_L0": (12, 9, [2, 2], "Ez", 0.001, 100.0, 1e-4),
    }
    small = {}
    for name, (Nx, Ny, npml, pol, dl, om, L0) in cases.items():
        eps = 1 + 11 * rng.random((Nx, Ny))
        sim = Simulation(om, eps, dl, npml, pol, L0=L0)
        A = canon(sim.A)
        small[f"{name}_args"] = np.array([Nx, Ny, npml[0], npml[1], dl, om, L0, 0 if pol == "Ez" else 1])
        small[f"{name}_eps"] = eps
        small[f"{name}_indptr"] = A.indptr
        small[f"{name}_indices"] = A.indices
        small[f"{name}_data"] = A.data
        for dn, D in sim.derivs.items():
            small[f"{name}_{dn}"] = canon(D).data
        src = np.zeros((Nx, Ny))
        src[Nx // 2, Ny // 3] = 1.0
        src[Nx // 3, Ny // 2] = -0.5
        sim.src = src
        f = sim.solve_fields(solver="scipy")
        small[f"{name}_src"] = src
        for fi, fv in zip(("f1", "f2", "f3"), f):
            small[f"{name}_{fi}"] = fv
        if pol == "Hz":
            A2, _ = construct_A(om, sim.xrange, sim.yrange, eps, npml, pol, L0, averaging=False)
            small[f"{name}_noavg_data"] = canon(A2).data
            f = sim.solve_fields(solver="scipy", averaging=False)
            small[f"{name}_noavg_f1"] = f[0]
            small[f"{name}_noavg_f2"] = f[1]
    np.savez_compressed(OUT / "small_ops.npz", **small)

    # 3. the 200x200 Ez point-source problem (eps 12 square)
    N = 200
    eps = np.ones((N, N))
    eps[80:120, 80:120] = 12
    sim = Simulation(omega155, eps, 0.02, [15, 15], "Ez")
    sim.src[100, 100] = 1
    A = canon(sim.A)
    Hx, Hy, Ez = sim.solve_fields(solver="scipy")
    rows = np.arange(0, N * N, 37)
    g = {
        "rows": rows,
        "row_indices": np.stack([A.indices[A.indptr[r]:A.indptr[r + 1]] for r in rows]),
        "row_data": np.stack([A.data[A.indptr[r]:A.indptr[r + 1]] for r in rows]),
        "data_abs_sum": np.abs(A.data).sum(),
        "sample": np.arange(0, N * N, 5),
        "Hx": Hx.reshape(-1)[::5], "Hy": Hy.reshape(-1)[::5], "Ez": Ez.reshape(-1)[::5],
        "norms": np.array([np.linalg.norm(Hx), np.linalg.norm(Hy), np.linalg.norm(Ez)]),
        "relres": np.linalg.norm(sim.A @ Ez.reshape(-1) - 1j * omega155 * sim.src.reshape(-1))
        / np.linalg.norm(1j * omega155 * sim.src.reshape(-1)),
    }
    np.savez_compressed(OUT / "ez200.npz", **g)

    # 4. Hz piecewise-constant blocks (the 2048^2 workload's family at 128^2)
    N = 128
    r0 = np.random.default_rng(0)
    eps = np.kron(r0.choice([1.0, 12.25], size=(N // 16, N // 16)), np.ones((16, 16)))
    sim = Simulation(omega155, eps, 0.01, [20, 20], "Hz")
    sim.src[30, :] = 1
    Ex, Ey, Hz = sim.solve_fields(solver="scipy")
    np.savez_compressed(OUT / "hz128_blocks.npz", eps=eps, Ex=Ex, Ey=Ey, Hz=Hz)

    # 5. mode source: the ridge waveguide of the examples notebook (Ez) and
    #    an Hz variant; W_in, E2_in and the inserted source line.  The
    #    reference's slice operator and eigenpair are captured by wrapping
    #    the solver_eigs it calls.
    import fdfdpy.source.mode as M
    captured = []
    orig_eigs = M.solver_eigs

    def recording_eigs(A, Neigs, guess_value=0, guess_vector=None, timing=False):
        vals, vecs = orig_eigs(A, Neigs, guess_value=guess_value, guess_vector=guess_vector, timing=timing)
        captured.append((A.toarray(), guess_value, vals.copy(), vecs.copy()))  # insert_mode scales vecs in place
        return vals, vecs

    M.solver_eigs = recording_eigs
    md = {}
    for pol in ("Ez", "Hz"):
        om = 2 * np.pi * 200e12
        eps = np.ones((600, 200))
        eps[:, 90:110] = 12.25
        sim = Simulation(om, eps, 0.01, [15, 15], pol)
        sim.add_mode(3.5, "x", [20, 100], 60, scale=10)
        if pol == "Ez":
            sim.setup_modes()
            md["ez_W_in"] = sim.W_in
            md["ez_E2_in"] = sim.E2_in
        else:
            # E2_in reads fields['Ez'] (mode.py:59-60), which the Hz branch
            # never fills, so only the source insertion is recorded for Hz.
            sim.modes[0].insert_mode(sim, sim.src)
        md[f"{pol.lower()}_src_line"] = sim.src[20, 70:130].copy()
        A1, sig, vals, vecs = captured[-1]
        md[f"{pol.lower()}_A1"] = A1
        md[f"{pol.lower()}_sigma"] = sig
        md[f"{pol.lower()}_eigval"] = vals
        md[f"{pol.lower()}_eigvec"] = vecs
    # a slice normal to y (its grid average runs along the slice)
    eps = np.ones((200, 300))
    eps[90:110, :] = 12.25
    sim = Simulation(2 * np.pi * 200e12, eps, 0.01, [15, 15], "Hz")
    sim.add_mode(3.5, "y", [100, 20], 60, scale=2)
    sim.modes[0].insert_mode(sim, sim.src)
    A1, sig, vals, vecs = captured[-1]
    md["hzy_A1"], md["hzy_sigma"], md["hzy_eigval"], md["hzy_eigvec"] = A1, sig, vals, vecs
    md["hzy_src_line"] = sim.src[70:130, 20].copy()
    M.solver_eigs = orig_eigs
    np.savez_compressed(OUT / "modes.npz", **md)

    kerr_golden()
    print("golden vectors written to", OUT)


def kerr_golden():
    """Kerr solves of the reference (solve_fields_nl -> newton_solve /
    born_solve, nonlinear_solvers.py:13-115; its complex-to-real Jacobian
    solves through the pyMKL shim, i.e. exact SuperLU): a 48 x 40 Ez grid
    with random eps, a 16 x 16 Kerr region and a point source.  Newton at
    amplitude 3e3 (eps_nl reaches ~10), Born at 3e2 (where the fixed point
    contracts)."""
    from fdfdpy import Simulation
    from fdfdpy.constants import C_0
    rng = np.random.default_rng(2)
    Nx, Ny, dl, chi = 48, 40, 0.02, 2.8e-18
    omega = 2 * np.pi * C_0 / 1.55e-6
    eps = 1 + 11 * rng.random((Nx, Ny))
    region = np.zeros((Nx, Ny))
    region[16:32, 12:28] = 1
    out = {"eps": eps, "region": region, "omega": omega, "dl": dl, "chi": chi, "npml": np.array([6, 6])}
    for solver, amp, iters in (("newton", 3e3, 50), ("born", 3e2, 200)):
        sim = Simulation(omega, eps, dl, [6, 6], "Ez")
        sim.src[10, 20] = amp
        sim.add_nl(chi, region)
        _, _, Ez, conv = sim.solve_fields_nl(solver_nl=solver, conv_threshold=1e-12, max_num_iter=iters)
        out[f"{solver}_amp"] = amp
        out[f"{solver}_Ez"] = Ez
        out[f"{solver}_conv"] = np.asarray(conv).reshape(-1)
    np.savez_compressed(OUT / "kerr48.npz", **out)


def kerr_sweep_golden(N=128, n_sample=2048):
    """The Kerr Newton workload (Ez, dl 0.02, NPML [20, 20], a centred
    square of eps 12 and chi3 2.8e-18 covering 400/1024 of the side, point
    source at (200/1024, 1/2) of the grid, amplitudes logspace(2, 5, 8)) at
    N x N, solved by the reference's own solve_fields_nl (Newton, its
    complex-to-real Jacobian solves through the exact-LU shim), 50
    iterations at most, threshold 1e-10.  Stored per amplitude: the
    convergence history and sampled entries (and the norm) of the final Ez."""
    from fdfdpy import Simulation
    from fdfdpy.constants import C_0
    omega = 2 * np.pi * C_0 / 1.55e-6
    r = N * 400 // 1024
    c0 = (N - r) // 2
    eps = np.ones((N, N))
    eps[c0:c0 + r, c0:c0 + r] = 12
    region = np.zeros((N, N))
    region[c0:c0 + r, c0:c0 + r] = 1
    amps = np.logspace(2, 5, 8)
    sample = np.sort(np.random.default_rng(3).choice(N * N, size=n_sample, replace=False))
    out = {"N": N, "amps": amps, "sample": sample, "src_ij": np.array([N * 200 // 1024, N // 2])}
    for k, a in enumerate(amps):
        sim = Simulation(omega, eps, 0.02, [20, 20], "Ez")
        sim.src[N * 200 // 1024, N // 2] = a
        sim.add_nl(2.8e-18, region)
        _, _, Ez, conv = sim.solve_fields_nl(solver_nl="newton", conv_threshold=1e-10, max_num_iter=50)
        out[f"conv_{k}"] = np.asarray(conv).reshape(-1)
        out[f"Ez_{k}"] = Ez.reshape(-1)[sample]
        out[f"norm_{k}"] = np.linalg.norm(Ez)
    np.savez_compressed(OUT / f"kerr{N}_sweep.npz", **out)


def design_golden():
    """Simulation.init_design_region of the reference (simulation.py:344-369)
    for each style on a small grid with a random eps_r and design region;
    numpy's global RNG is seeded with 5 before each call ('random' draws
    from it)."""
    from fdfdpy import Simulation
    from fdfdpy.constants import C_0
    rng = np.random.default_rng(9)
    eps = 1 + 3 * rng.random((20, 16))
    region = np.zeros((20, 16))
    region[5:14, 4:11] = 1
    out = {"eps": eps, "region": region}
    for style in ("full", "halfway", "empty", "random", "other"):
        sim = Simulation(2 * np.pi * C_0 / 1.55e-6, eps.copy(), 0.02, [3, 3], "Ez")
        np.random.seed(5)
        sim.init_design_region(region, 7.5, style=style)
        out[style] = np.array(sim.eps_r)
    np.savez_compressed(OUT / "design.npz", **out)


def projection_vectors(n, count, seed=2048):
    """`count` complex Gaussian vectors of length n with E|g.v|^2 = ||v||^2,
    generated one after the other from numpy's PCG64 stream (identical on
    every platform), so a test can rebuild them to estimate a field error
    from projections."""
    rng = np.random.default_rng(seed)
    for _ in range(count):
        g = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        yield g / np.sqrt(2.0)


def hz2048_golden(n_sample=4096, n_proj=8, refine_steps=3):
    """The large single solve (Hz, 2048 x 2048, dl 0.01, NPML [20, 20],
    16 x 16 blocks of {1, 12.25} from seed 0, src[30, :] = 1) by the
    reference's own solve_fields (default solver path: the exact-LU shim),
    then `refine_steps` FP64 iterative-refinement steps with that same
    factor; the secondary fields of the refined Hz follow the reference's
    field recovery (simulation.py:133-160).  Stored: sampled entries of the
    raw and refined fields, their norms and relative residuals, and the
    projections of the refined fields on seeded Gaussian vectors."""
    import time
    from fdfdpy import Simulation
    from fdfdpy.constants import C_0, EPSILON_0
    from fdfdpy.linalg import grid_average
    N, dl, npml = 2048, 0.01, [20, 20]
    omega = 2 * np.pi * C_0 / 1.55e-6
    r0 = np.random.default_rng(0)
    eps = np.kron(r0.choice([1.0, 12.25], size=(N // 16, N // 16)), np.ones((16, 16)))
    t0 = time.time()
    sim = Simulation(omega, eps, dl, npml, "Hz")
    sim.src[30, :] = 1
    Ex, Ey, Hz = sim.solve_fields()
    t_solve = time.time() - t0
    A, lu = LAST_FACTOR
    b = (1j * omega * sim.src).reshape(-1).astype(np.complex128)
    bn = np.linalg.norm(b)
    x = Hz.reshape(-1).copy()
    res = [np.linalg.norm(b - A @ x) / bn]
    for _ in range(refine_steps):
        x = x + lu.solve(b - A @ x)
        res.append(np.linalg.norm(b - A @ x) / bn)
    D = sim.derivs
    e0 = EPSILON_0 * sim.L0
    ex_avg = grid_average(e0 * eps, 'x').reshape(-1)
    ey_avg = grid_average(e0 * eps, 'y').reshape(-1)
    Exr = 1 / 1j / omega * ((1 / ey_avg) * D['Dyb'].dot(x))
    Eyr = -1 / 1j / omega * ((1 / ex_avg) * D['Dxb'].dot(x))
    n = N * N
    sample = np.sort(np.random.default_rng(7).choice(n, size=n_sample, replace=False))
    out = {"N": N, "dl": dl, "npml": np.array(npml), "omega": omega, "sample": sample,
           "raw_Ex": Ex.reshape(-1)[sample], "raw_Ey": Ey.reshape(-1)[sample], "raw_Hz": Hz.reshape(-1)[sample],
           "raw_norms": np.array([np.linalg.norm(Ex), np.linalg.norm(Ey), np.linalg.norm(Hz)]),
           "Ex": Exr[sample], "Ey": Eyr[sample], "Hz": x[sample],
           "norms": np.array([np.linalg.norm(Exr), np.linalg.norm(Eyr), np.linalg.norm(x)]),
           "relres": np.array(res), "solve_s": t_solve,
           "raw_vs_refined": np.array([np.linalg.norm(Ex.reshape(-1) - Exr) / np.linalg.norm(Exr),
                                       np.linalg.norm(Ey.reshape(-1) - Eyr) / np.linalg.norm(Eyr),
                                       np.linalg.norm(Hz.reshape(-1) - x) / np.linalg.norm(x)])}
    proj = np.zeros((n_proj, 3), dtype=np.complex128)
    for k, g in enumerate(projection_vectors(n, n_proj)):
        proj[k] = [g @ Exr, g @ Eyr, g @ x]
    out["proj"] = proj
    np.savez_compressed(OUT / "hz2048.npz", **out)
    print("hz2048: solve %.1f s, residuals %s" % (t_solve, res))


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="path of the reference checkout")
    ap.add_argument("--only", default=None, choices=["kerr", "hz2048", "kerr_sweep", "design"])
    a = ap.parse_args()
    if a.reference:
        REF = a.reference
    if a.only:
        install_shims()
        import warnings
        warnings.simplefilter("ignore")
        {"kerr": kerr_golden, "hz2048": hz2048_golden, "kerr_sweep": kerr_sweep_golden,
         "design": design_golden}[a.only]()
        print("golden vectors written to", OUT)
    else:
        main()
