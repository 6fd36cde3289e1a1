"""The C-ABI library: it loads, exports every entry point the public header
declares, and rejects bad arguments with status codes (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from fdfdpy_gb300 import _native, build
    if not _native._LIB_PATH.exists():
        build.build()
    return _native.lib()


def declared_functions():
    src = (ROOT / "include" / "fdfd_gb300.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fdfd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("fdfd_assemble_csr", "fdfd_residual", "fdfd_fields", "fdfd_symbolic_create",
                 "fdfd_factor_create", "fdfd_factor_numeric", "fdfd_solve_refined",
                 "fdfd_adjoint_grad_eps", "fdfd_pml_sfactors"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from fdfdpy_gb300 import _native
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_version_and_errors(lib):
    from fdfdpy_gb300 import _native as N
    assert lib.fdfd_version() == 1
    h = C.c_void_p()
    assert lib.fdfd_symbolic_create(0, 5, 16, C.byref(h)) == N.FDFD_ERR_BAD_ARG
    assert b"grid" in lib.fdfd_last_error()
    assert lib.fdfd_assemble_csr(None, None, None, None, None) == N.FDFD_ERR_BAD_ARG
    op = N.Operator()
    op.Nx, op.Ny, op.pol = 2, 8, 0
    assert lib.fdfd_residual(C.byref(op), None, None, None, 1, None) == N.FDFD_ERR_BAD_ARG
    assert b"Nx >= 3" in lib.fdfd_last_error()
    op.Nx, op.pol = 8, 7
    assert lib.fdfd_fields(C.byref(op), None, None, None, None) == N.FDFD_ERR_BAD_ARG
    assert lib.fdfd_factor_bytes(None, 0, 1, None) == N.FDFD_ERR_BAD_ARG


def test_factor_bytes_host_only(lib):
    from fdfdpy_gb300 import engine
    sym = engine.Symbolic(64, 64)
    b128 = engine.Factor.bytes_needed(sym, "c128")
    b64 = engine.Factor.bytes_needed(sym, "c64")
    assert b64 < b128 and b128 > sym.info.pool_entries * 16


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-device path")
def test_no_cpu_fallback():
    from fdfdpy_gb300 import Simulation, engine, _native as N
    with pytest.raises(N.FDFDError):
        Simulation(1e15, np.ones((8, 8)), 0.02, [2, 2], "Ez")
    sym = engine.Symbolic(8, 8)
    h = C.c_void_p()
    assert N.lib().fdfd_factor_create(sym.handle, 0, 1, C.byref(h)) == N.FDFD_ERR_NO_DEVICE


def test_reference_input_checks():
    from fdfdpy_gb300 import Simulation
    # the reference asserts on these before any operator is built (simulation.py:249-256)
    with pytest.raises(AssertionError):
        Simulation(1e15, np.ones((8, 8)), 0.02, [2, 2], "Ex")
    with pytest.raises(AssertionError):
        Simulation(1e15, np.ones((8, 8)), 0.02, [-1, 2], "Ez")
    with pytest.raises(AssertionError):
        Simulation(1e15, np.ones((8, 8)), 0.02, [2, 2, 2], "Ez")
    with pytest.raises(AssertionError):
        Simulation(1e15, np.ones((8, 8)), 0.02, [2, 2], "Ez", L0=-1)
