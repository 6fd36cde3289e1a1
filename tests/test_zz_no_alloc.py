"""The allocation-free column-norm entry point (fdfd_norms_noalloc).

It exists for callers that cannot allocate device memory when they call
in -- for example a process whose GPU memory is already held by its own
allocator under a fixed budget.  This test calls it through the C ABI
twice in a row (the fixed scratch keeps the first call's contents) and
checks both results against the allocating entry point, fdfd_norms, to the
tolerance used for the reductions elsewhere (1e-13 relative).  Around each
allocation-free call it also checks that no device memory was allocated:
torch's caching allocator and the CUDA runtime's default memory pool (the
one cudaMallocAsync draws from) hold no more memory after the call than
before.  The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _norms(fn, v, n, ncol):
    from fdfdpy_gb300 import _native as N
    out = (C.c_double * ncol)()
    st = torch.cuda.current_stream().cuda_stream
    rc = getattr(N.lib(), fn)(C.c_void_p(v.data_ptr()), n, ncol, out, C.c_void_p(st))
    assert rc == N.FDFD_OK, N.lib().fdfd_last_error()
    return np.array(out[:])


def _device_memory_in_use():
    """(torch allocated, torch reserved, default-pool used, default-pool
    reserved) bytes on the current device."""
    rt = C.CDLL("libcudart.so.13")             # the runtime the library itself loaded
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), torch.cuda.current_device()) == 0
    used, reserved = C.c_uint64(), C.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, 0x7, C.byref(used)) == 0       # UsedMemCurrent
    assert rt.cudaMemPoolGetAttribute(pool, 0x5, C.byref(reserved)) == 0   # ReservedMemCurrent
    return (torch.cuda.memory_allocated(), torch.cuda.memory_reserved(), used.value, reserved.value)


def test_noalloc_norms_match_allocating_entry_point_twice():
    from fdfdpy_gb300 import _native as N
    N.lib()
    rng = np.random.default_rng(17)
    cases = [(250007, 3), (4097, 8)]           # two calls in a row, different shapes
    for n, ncol in cases:
        h = rng.standard_normal((ncol, n)) + 1j * rng.standard_normal((ncol, n))
        v = torch.from_numpy(h).cuda()
        torch.cuda.synchronize()
        before = _device_memory_in_use()
        got = _norms("fdfd_norms_noalloc", v, n, ncol)
        torch.cuda.synchronize()
        after = _device_memory_in_use()
        assert after[0] == before[0] and after[2] == before[2], (before, after)
        assert after[1] <= before[1] and after[3] <= before[3], (before, after)
        want = _norms("fdfd_norms", v, n, ncol)
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=0)
        np.testing.assert_allclose(got, np.linalg.norm(h, axis=1), rtol=1e-13)


def test_noalloc_rejects_too_many_columns():
    from fdfdpy_gb300 import _native as N
    v = torch.zeros(9 * 16, dtype=torch.complex128, device="cuda")
    out = (C.c_double * 9)()
    rc = N.lib().fdfd_norms_noalloc(C.c_void_p(v.data_ptr()), 16, 9, out, None)
    assert rc == N.FDFD_ERR_BAD_ARG
    assert b"at most 8 columns" in N.lib().fdfd_last_error()
