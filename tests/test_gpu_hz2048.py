"""The large single solve (Hz, 2048 x 2048, dl 0.01, NPML [20, 20], 16 x 16
blocks of {1, 12.25} from seed 0, src[30, :] = 1) against the reference's
own solution of it (tests/golden/hz2048.npz: the reference's solve_fields
through its default solver path with an exact LU, then three FP64
refinement steps with that factor; generated by tests/golden/make_golden.py
--only hz2048).  The full fields (67 MB each) are not stored: the fixture
holds 4096 sampled entries of each field, the field norms, and projections
of the fields on eight seeded complex Gaussian vectors g_k, whose
differences estimate the full-field error (E|g.v|^2 = ||v||^2).

Bars: complex128 factor (refined to 1e-12) <= 1e-10 relative; complex64
factor with tensor-core Schur updates, refined to a residual of 1e-10,
<= 1e-8 relative (field error bounded by cond(A) x residual)."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "hz2048.npz"


def _vectors(n, count, seed=2048):
    rng = np.random.default_rng(seed)
    for _ in range(count):
        g = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        yield g / np.sqrt(2.0)


@pytest.mark.skipif(not GOLD.exists(), reason="fixture not generated")
def test_hz2048_matches_reference_solution():
    from fdfdpy_gb300 import Simulation
    from fdfdpy_gb300.constants import C_0
    g = np.load(GOLD)
    N = int(g["N"])
    omega = 2 * np.pi * C_0 / 1.55e-6
    assert omega == g["omega"]
    rng = np.random.default_rng(0)
    eps = np.kron(rng.choice([1.0, 12.25], size=(N // 16, N // 16)), np.ones((16, 16)))
    assert g["relres"][-1] < 1e-12          # the refined reference solution
    s = g["sample"]
    nproj = g["proj"].shape[0]
    vecs = list(_vectors(N * N, nproj))
    for prec, tol in (("c128", 1e-10), ("c64tc", 1e-8)):
        sim = Simulation(omega, eps, 0.01, [20, 20], "Hz")
        sim.src[30, :] = 1
        fields = [f.reshape(-1) for f in sim.solve_fields(precision=prec)]
        assert sim.last_solve_stats["rel_residual"] <= (1e-12 if prec == "c128" else 1e-10)
        for j, name in enumerate(("Ex", "Ey", "Hz")):
            samp = np.linalg.norm(fields[j][s] - g[name]) / np.linalg.norm(g[name])
            proj = np.array([v @ fields[j] for v in vecs])
            est = np.linalg.norm(proj - g["proj"][:, j]) / np.linalg.norm(g["proj"][:, j])
            nrm = abs(np.linalg.norm(fields[j]) - g["norms"][j]) / g["norms"][j]
            assert samp <= tol and est <= tol and nrm <= tol, (prec, name, samp, est, nrm)
        del sim
