"""Failure surfacing of the engine's bounded device-side waits.

The cooperative substitutions (grid barrier, published panel values) give up
after a bounded number of polls and the call returns FDFD_ERR_TIMEOUT
(DeviceTimeout in Python) instead of hanging.  The test shortens the limit
to one poll so that the waits run out (nothing is broken on purpose: every
wait still ends, the kernels return and the context stays usable), checks
the status, then restores the default limit and checks that the next solve
on the same factor succeeds.  No wait of the tensor-core Schur kernel is
forced to run out (its copies and MMAs could still be in flight)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _blocks(N, seed=0):
    rng = np.random.default_rng(seed)
    return np.kron(rng.choice([1.0, 12.25], size=(N // 16, N // 16)), np.ones((16, 16)))


def test_wait_limit_reports_timeout_then_default_limit_solves():
    import torch
    from fdfdpy_gb300 import engine, _native as NAT
    from fdfdpy_gb300.constants import C_0
    N = 512
    om = 2 * np.pi * C_0 / 1.55e-6
    op = engine.DeviceOperator(om, _blocks(N), N * 0.01, N * 0.01, [20, 20], "Hz", 1e-6)
    sym = engine.symbolic_for(N, N)
    assert sym.info.max_p > 64          # the top levels run the cooperative substitutions
    fac = engine.Factor(sym, "c64").numeric(op)
    src = np.zeros((N, N))
    src[30, :] = 1.0
    b = engine.as_c128(1j * om * src).reshape(-1)
    fac.set_wait_limit(1)
    with pytest.raises(NAT.DeviceTimeout):
        fac.solve(b, tol=1e-10, max_iter=30, raise_on_fail=True)
    with pytest.raises(NAT.DeviceTimeout):
        fac.apply_inverse(b)
    fac.set_wait_limit(None)
    x = fac.solve(b, tol=1e-10, max_iter=30, raise_on_fail=True)
    r = op.residual(x, b)
    assert float(torch.linalg.vector_norm(r) / torch.linalg.vector_norm(b)) <= 1e-10
    # the device is still usable: a fresh factor of the same operator agrees
    x2 = engine.Factor(sym, "c64").numeric(op).solve(b, tol=1e-10, max_iter=30, raise_on_fail=True)
    assert float(torch.linalg.vector_norm(x2 - x) / torch.linalg.vector_norm(x)) <= 1e-8


def test_wait_limit_argument_checks():
    from fdfdpy_gb300 import engine, _native as NAT
    import ctypes as C
    sym = engine.symbolic_for(64, 64)
    fac = engine.Factor(sym, "c64")
    assert NAT.lib().fdfd_factor_set_wait_limit(fac.handle, 0) == NAT.FDFD_ERR_BAD_ARG
    assert NAT.lib().fdfd_factor_set_wait_limit(fac.handle, -1) == NAT.FDFD_OK
    assert NAT.lib().fdfd_factor_set_wait_limit(C.c_void_p(), 5) == NAT.FDFD_ERR_BAD_ARG
