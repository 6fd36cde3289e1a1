"""ctypes binding of the engine's C ABI (include/fdfd_gb300.h).

The shared library is built in-tree by ``fdfdpy_gb300.build`` (or
``__graft_entry__.build()``).  There is no fallback: if the library is
missing, every GPU entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libfdfd_gb300.so"

FDFD_OK = 0
FDFD_ERR_BAD_ARG = 1
FDFD_ERR_OOM = 2
FDFD_ERR_CUDA = 3
FDFD_ERR_SINGULAR_PIVOT = 4
FDFD_ERR_NOT_CONVERGED = 5
FDFD_ERR_NO_DEVICE = 6
FDFD_ERR_TIMEOUT = 7

POL = {"Ez": 0, "Hz": 1}
PREC = {"c128": 0, "c64": 1, "c64tc": 2}


class FDFDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[fdfd status {code}] {msg}")
        self.code = code


class NotConverged(FDFDError):
    pass


class DeviceTimeout(FDFDError):
    """A bounded device-side wait ran out; the call's result is not valid."""


class Operator(C.Structure):
    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("pol", C.c_int32), ("averaging", C.c_int32),
        ("omega", C.c_double), ("L0", C.c_double), ("xlen", C.c_double), ("ylen", C.c_double),
        ("eps", C.c_void_p), ("eps_add", C.c_void_p), ("diag_add", C.c_void_p),
        ("inv_sxf", C.c_void_p), ("inv_sxb", C.c_void_p), ("inv_syf", C.c_void_p),
        ("inv_syb", C.c_void_p), ("stencil", C.c_void_p),
    ]


class SymbolicInfo(C.Structure):
    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("n_fronts", C.c_int32), ("n_levels", C.c_int32),
        ("sum_m", C.c_int64), ("pool_entries", C.c_int64), ("factor_entries", C.c_int64),
        ("factor_flops", C.c_double), ("max_m", C.c_int32), ("max_p", C.c_int32),
    ]


class FactorStats(C.Structure):
    _fields_ = [
        ("tiny_pivots", C.c_int32), ("refine_iters", C.c_int32), ("rel_residual", C.c_double),
        ("factor_ms", C.c_double), ("solve_ms", C.c_double), ("tc_errors", C.c_int32), ("pad", C.c_int32),
    ]


P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
D = C.c_double
POP = C.POINTER(Operator)

# name -> (restype, argtypes)
SIGNATURES = {
    "fdfd_last_error": (C.c_char_p, []),
    "fdfd_version": (C.c_int, []),
    "fdfd_pml_sfactors": (C.c_int, [I32, I32, D, D, D, P, P, P]),
    "fdfd_assemble_csr": (C.c_int, [POP, P, P, P, P]),
    "fdfd_assemble_deriv_csr": (C.c_int, [POP, I32, P, P, P, P]),
    "fdfd_residual": (C.c_int, [POP, P, P, P, I32, P]),
    "fdfd_apply": (C.c_int, [POP, P, P, I32, I32, P]),
    "fdfd_fields": (C.c_int, [POP, P, P, P, P]),
    "fdfd_adjoint_grad_eps": (C.c_int, [POP, P, P, P, P]),
    "fdfd_mode_stencil": (C.c_int, [I32, I32, I32, P, D, D, D, D, P, P]),
    "fdfd_norms": (C.c_int, [P, I64, I32, P, P]),
    "fdfd_kerr_assemble": (C.c_int, [I64, P, P, P, D, I32, D, D, D, I32, P, P, P, P, P, P]),
    "fdfd_flux_probe": (C.c_int, [I32, I32, I32, I32, I32, I32, I32, D, P, P, P, P]),
    "fdfd_norms_noalloc": (C.c_int, [P, I64, I32, P, P]),
    "fdfd_symbolic_create": (C.c_int, [I32, I32, I32, C.POINTER(P)]),
    "fdfd_symbolic_create_batch": (C.c_int, [I32, I32, I32, I32, C.POINTER(P)]),
    "fdfd_symbolic_info_get": (C.c_int, [P, C.POINTER(SymbolicInfo)]),
    "fdfd_symbolic_export": (C.c_int, [P, I32, P]),
    "fdfd_symbolic_destroy": (None, [P]),
    "fdfd_factor_bytes": (C.c_int, [P, I32, I32, C.POINTER(I64)]),
    "fdfd_factor_create": (C.c_int, [P, I32, I32, C.POINTER(P)]),
    "fdfd_factor_numeric": (C.c_int, [P, POP, P]),
    "fdfd_factor_solve": (C.c_int, [P, P, P, I32, I32, P]),
    "fdfd_solve_refined": (C.c_int, [P, POP, P, P, I32, I32, D, I32, P]),
    "fdfd_solve_gmres": (C.c_int, [P, POP, P, P, I32, D, I32, I32, P]),
    "fdfd_factor_numeric_batch": (C.c_int, [P, POP, I32, P]),
    "fdfd_solve_refined_batch": (C.c_int, [P, P, P, I32, D, I32, P, P]),
    "fdfd_factor_stats_get": (C.c_int, [P, C.POINTER(FactorStats)]),
    "fdfd_factor_coef_get": (C.c_int, [P, P, P]),
    "fdfd_factor_set_pivot_tol": (C.c_int, [P, D]),
    "fdfd_factor_set_fused_limit": (C.c_int, [P, I32]),
    "fdfd_factor_set_wait_limit": (C.c_int, [P, I64]),
    "fdfd_factor_set_graphs": (C.c_int, [P, I32]),
    "fdfd_factor_destroy": (None, [P]),
    "fdfd_profile_enable": (C.c_int, [I32]),
    "fdfd_profile_reset": (C.c_int, []),
    "fdfd_profile_read": (C.c_int, [I32, P, P]),
}

PROFILE_CLASSES = ("assemble", "extend_add", "lu_diag", "trsm", "schur", "solve_fwd", "solve_bwd", "other",
                   "schur_simt")


def profile_read():
    """{class: (ms, launches)} accumulated since the last reset."""
    nc = len(PROFILE_CLASSES)
    ms = (C.c_double * nc)()
    cnt = (C.c_int64 * nc)()
    call("fdfd_profile_read", nc, ms, cnt)
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PROFILE_CLASSES)}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise FDFDError(-1, f"{_LIB_PATH.name} is not built; run fdfdpy_gb300.build.build() "
                                "(the engine has no CPU fallback)")
        L = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code, what=""):
    if code == FDFD_OK:
        return
    msg = lib().fdfd_last_error().decode(errors="replace")
    if code == FDFD_ERR_NOT_CONVERGED:
        raise NotConverged(code, msg)
    if code == FDFD_ERR_TIMEOUT:
        raise DeviceTimeout(code, f"{what}: {msg}" if what else msg)
    raise FDFDError(code, f"{what}: {msg}" if what else msg)


def call(name, *args):
    check(getattr(lib(), name)(*args), name)
