"""The tcgen05 (tensor-core, 3xTF32) Schur update of the complex64 factor:
same refined solutions as the SIMT complex64 factor and the oracle, no
timed-out tiles, and a factor error of FP32 level (refinement converges in
as few steps as with the SIMT kernel, plus at most two)."""
import numpy as np
import pytest

from oracle import fdfd_oracle as O

pytestmark = pytest.mark.gpu
OMEGA = 2 * np.pi * O.C_0 / 1.55e-6


@pytest.mark.parametrize("N,M,pol", [(200, 200, "Ez"), (300, 260, "Hz"), (520, 130, "Ez")])
def test_tensor_core_factor_matches_simt_and_oracle(N, M, pol):
    from fdfdpy_gb300 import engine
    rng = np.random.default_rng(N + M)
    eps = np.kron(rng.choice([1.0, 12.25], size=(N // 10, M // 10)), np.ones((10, 10)))
    op = engine.DeviceOperator(OMEGA, eps, N * 0.02, M * 0.02, [15, 15], pol, 1e-6)
    sym = engine.symbolic_for(N, M)
    assert sym.info.max_m >= 512  # the tensor-core levels are exercised
    b = rng.standard_normal(N * M) + 1j * rng.standard_normal(N * M)
    xs, its = {}, {}
    for prec in ("c64", "c64tc"):
        fac = engine.Factor(sym, prec).numeric(op)
        x1 = fac.apply_inverse(b).cpu().numpy()
        x = fac.solve(b, tol=1e-10, max_iter=40, raise_on_fail=True).cpu().numpy()
        st = fac.stats()
        assert st["tc_errors"] == 0 and st["rel_residual"] <= 1e-10
        xs[prec], its[prec] = (x1, x), st["refine_iters"]
    A = O.construct_A(OMEGA, N * 0.02, M * 0.02, eps, [15, 15], pol, 1e-6)
    xr = O.solve(A, b)
    for prec in ("c64", "c64tc"):
        assert np.linalg.norm(xs[prec][1] - xr) / np.linalg.norm(xr) < 1e-8
    # one unrefined application: FP32-level agreement between the two kernels
    d = np.linalg.norm(xs["c64tc"][0] - xs["c64"][0]) / np.linalg.norm(xs["c64"][0])
    e = np.linalg.norm(xs["c64"][0] - xr) / np.linalg.norm(xr)
    assert d <= max(10 * e, 1e-5), (d, e)
    assert its["c64tc"] <= its["c64"] + 2
