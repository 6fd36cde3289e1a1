"""Mode sources on the GPU (fdfdpy/source/mode.py): slice operator, the
shift-invert eigenpair from the engine's factor, the inserted source line
(up to ARPACK's arbitrary global sign) and the input power W_in of the
examples notebook's ridge waveguide (published value 0.0016689050319357455,
notebooks/Examples.ipynb cell 7)."""
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
OM = 2 * np.pi * 200e12


def _wg(tag):
    if tag == "hzy":
        eps = np.ones((200, 300))
        eps[90:110, :] = 12.25
        return eps, "Hz", ("y", [100, 20], 60, 2), (slice(70, 130), 20)
    eps = np.ones((600, 200))
    eps[:, 90:110] = 12.25
    return eps, ("Ez" if tag == "ez" else "Hz"), ("x", [20, 100], 60, 10), (20, slice(70, 130))


@pytest.mark.parametrize("tag,average", [("ez", False), ("hz", False), ("hzy", True)])
def test_slice_operator_and_eigenpair(tag, average):
    from fdfdpy_gb300 import engine
    m = np.load(GOLD / "modes.npz")
    eps, pol, _, sl = _wg(tag)
    e_sl = eps[sl]
    op = engine.StencilOperator.mode_slice(pol, e_sl, OM, 0.01, 1e-6, 0.0, average)
    n = e_sl.size
    dense = op.apply(torch.eye(n, dtype=torch.complex128)).cpu().numpy().T  # columns A e_k
    want = m[tag + "_A1"]
    assert np.max(np.abs(dense - want)) <= 1e-15 * np.max(np.abs(want))
    sigma = float(m[tag + "_sigma"])
    ops = engine.StencilOperator.mode_slice(pol, e_sl, OM, 0.01, 1e-6, sigma, average)
    vals, vecs = engine.shift_invert_eigs(ops, sigma, 1)
    assert abs(vals[0] - m[tag + "_eigval"][0]) <= 1e-10 * abs(vals[0])
    v = vecs[:, 0].cpu().numpy()
    w = m[tag + "_eigvec"][:, 0]
    ph = np.vdot(w, v) / abs(np.vdot(w, v))
    assert np.linalg.norm(v / ph - w) < 1e-8


@pytest.mark.parametrize("tag", ["ez", "hz", "hzy"])
def test_insert_mode_source_line(tag):
    from fdfdpy_gb300 import Simulation
    m = np.load(GOLD / "modes.npz")
    eps, pol, (d, c, w, scale), sl = _wg(tag)
    sim = Simulation(OM, eps, 0.01, [15, 15], pol)
    sim.add_mode(3.5, d, c, w, scale=scale)
    sim.modes[0].insert_mode(sim, sim.src)
    got, want = sim.src[sl], m[tag + "_src_line"]
    assert min(np.linalg.norm(got - want), np.linalg.norm(got + want)) <= 1e-9 * np.linalg.norm(want)
    assert np.count_nonzero(sim.src) == np.count_nonzero(want)


def test_waveguide_input_power_matches_notebook():
    from fdfdpy_gb300 import Simulation
    m = np.load(GOLD / "modes.npz")
    eps, pol, (d, c, w, scale), _ = _wg("ez")
    sim = Simulation(OM, eps, 0.01, [15, 15], "Ez")
    sim.add_mode(3.5, d, c, w, scale=scale)
    sim.setup_modes()
    assert abs(sim.W_in - 0.0016689050319357455) <= 1e-9 * 0.0016689050319357455
    assert abs(sim.E2_in - m["ez_E2_in"]) <= 1e-9 * abs(m["ez_E2_in"])
    Hx, Hy, Ez = sim.solve_fields()
    assert np.isfinite(Ez).all() and np.abs(Ez).max() > 0
