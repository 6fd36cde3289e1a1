"""Device-side objects of the engine: operators, symbolic analyses, factors.

Device memory for operator inputs and right-hand sides is held in torch
tensors (torch is used for allocation and streams only); every computation
is a call into the engine's CUDA library through its C ABI.  Nothing here
computes on the CPU besides O(1) bookkeeping; a machine without a CUDA
device gets an error, not a slower path.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as N
from .constants import DEFAULT_LEAF_AREA


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise N.FDFDError(N.FDFD_ERR_NO_DEVICE, "the FDFD engine needs a CUDA device (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def as_c128(x, shape=None) -> torch.Tensor:
    """Host/device array -> contiguous complex128 device tensor."""
    dev = device()
    if isinstance(x, torch.Tensor):
        # lazy conjugate / negative views must be materialised: the C ABI
        # reads raw memory
        t = x.to(device=dev, dtype=torch.complex128).resolve_conj().resolve_neg()
    else:
        a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
        t = torch.from_numpy(a).to(dev, non_blocking=False)
    t = t.contiguous()
    return t if shape is None else t.reshape(shape)


def to_host(*ts):
    """Device tensors -> numpy arrays through page-locked buffers from
    torch's caching host allocator (the copies run at link speed, with no
    staging copy on the host; a buffer is reused once the caller has dropped
    an earlier result).  Each tensor's copy runs on its own copy stream, so
    that several copies share the link at once."""
    pending = [to_host_start(t, slot=i) for i, t in enumerate(ts)]
    return [to_host_finish(p) for p in pending]


_copy_streams: dict = {}
_copy_lock = threading.Lock()


def to_host_start(t, slot=0):
    """Start the device -> host copy of t into a page-locked buffer on copy
    stream `slot` (of a few per device), after the work queued so far on the
    current stream, so that it runs beside the kernels queued next (t must
    not be written by them).  to_host_finish returns the numpy array."""
    cur = torch.cuda.current_stream()
    # copy streams of the caller's stream: callers on other streams (the
    # serving slots) do not queue behind each other's copies
    with _copy_lock:
        if len(_copy_streams) > 64:
            _copy_streams.clear()  # callers that come and go: torch's streams are pooled, none is destroyed
        pool = _copy_streams.setdefault((cur.device, cur.cuda_stream), [])
        while len(pool) <= slot:
            pool.append(torch.cuda.Stream(device=cur.device))
        st = pool[slot]
    st.wait_stream(cur)
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    with torch.cuda.stream(st):
        h.copy_(t, non_blocking=True)
    t.record_stream(st)
    ev = torch.cuda.Event()
    ev.record(st)
    return h, ev


def to_host_finish(pending):
    h, ev = pending
    ev.synchronize()
    return h.numpy()


def as_f64(x) -> torch.Tensor:
    dev = device()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float64).resolve_neg().contiguous()
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return torch.from_numpy(a).to(dev)


class DeviceOperator:
    """The PML-stretched operator of one (omega, eps_r, dl, NPML, pol, L0)
    on the device: eps_r, the four 1/s vectors (computed on the GPU) and the
    C-ABI operator struct pointing at them.  Mirrors the inputs of
    construct_A (fdfdpy/linalg.py:41-44)."""

    def __init__(self, omega, eps_r, xlen, ylen, NPML, pol, L0, averaging=True,
                 eps_add=None, diag_add=None):
        if pol not in N.POL:
            raise ValueError(f"Invalid polarization: {pol}")
        eps = eps_r if isinstance(eps_r, torch.Tensor) else np.asarray(eps_r, dtype=np.float64)
        if eps.ndim != 2:
            raise ValueError("eps_r must be a 2-D array")
        self.Nx, self.Ny = int(eps.shape[0]), int(eps.shape[1])
        if self.Nx < 3 or self.Ny < 3:
            raise ValueError("the GPU operator needs a grid of at least 3 x 3 cells")
        self.omega, self.L0, self.pol = float(omega), float(L0), pol
        self.xlen, self.ylen = float(xlen), float(ylen)
        self.NPML = [int(NPML[0]), int(NPML[1])]
        self.averaging = bool(averaging)
        self.eps = as_f64(eps).reshape(-1)
        self.eps_add = None if eps_add is None else as_f64(eps_add).reshape(-1)
        self.diag_add = None if diag_add is None else as_c128(diag_add).reshape(-1)
        dev = device()
        self.inv_s = [torch.empty(self.Nx, dtype=torch.complex128, device=dev),
                      torch.empty(self.Nx, dtype=torch.complex128, device=dev),
                      torch.empty(self.Ny, dtype=torch.complex128, device=dev),
                      torch.empty(self.Ny, dtype=torch.complex128, device=dev)]
        st = stream_ptr()
        N.call("fdfd_pml_sfactors", self.Nx, self.NPML[0], self.xlen, self.omega, self.L0,
               _ptr(self.inv_s[0]), _ptr(self.inv_s[1]), st)
        N.call("fdfd_pml_sfactors", self.Ny, self.NPML[1], self.ylen, self.omega, self.L0,
               _ptr(self.inv_s[2]), _ptr(self.inv_s[3]), st)

    @property
    def n(self):
        return self.Nx * self.Ny

    def struct(self, averaging=None, eps=None, eps_add="keep", diag_add="keep") -> N.Operator:
        op = N.Operator()
        op.Nx, op.Ny, op.pol = self.Nx, self.Ny, N.POL[self.pol]
        op.averaging = int(self.averaging if averaging is None else averaging)
        op.omega, op.L0, op.xlen, op.ylen = self.omega, self.L0, self.xlen, self.ylen
        op.eps = (self.eps if eps is None else eps).data_ptr()
        ea = self.eps_add if isinstance(eps_add, str) else eps_add
        da = self.diag_add if isinstance(diag_add, str) else diag_add
        op.eps_add = None if ea is None else ea.data_ptr()
        op.diag_add = None if da is None else da.data_ptr()
        op.inv_sxf, op.inv_sxb, op.inv_syf, op.inv_syb = (t.data_ptr() for t in self.inv_s)
        self._keep = (ea, da)
        return op

    def with_terms(self, eps_add=None, diag_add=None) -> "DeviceOperator":
        """Same operator with a diagonal Kerr term / complex diagonal added."""
        o = object.__new__(DeviceOperator)
        o.__dict__.update(self.__dict__)
        o.eps_add = None if eps_add is None else as_f64(eps_add).reshape(-1)
        o.diag_add = None if diag_add is None else as_c128(diag_add).reshape(-1)
        return o

    # ---- K1 -----------------------------------------------------------------
    def csr_device(self):
        dev = device()
        n = self.n
        indptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
        indices = torch.empty(5 * n, dtype=torch.int32, device=dev)
        data = torch.empty(5 * n, dtype=torch.complex128, device=dev)
        op = self.struct()
        N.call("fdfd_assemble_csr", C.byref(op), _ptr(indptr), _ptr(indices), _ptr(data), stream_ptr())
        return indptr, indices, data

    def csr(self) -> sp.csr_matrix:
        indptr, indices, data = self.csr_device()
        n = self.n
        return sp.csr_matrix((data.cpu().numpy(), indices.cpu().numpy(), indptr.cpu().numpy()),
                             shape=(n, n))

    def deriv_csr(self, which: str) -> sp.csr_matrix:
        code = {"Dxf": 0, "Dxb": 1, "Dyf": 2, "Dyb": 3}[which]
        dev = device()
        n = self.n
        indptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
        indices = torch.empty(2 * n, dtype=torch.int32, device=dev)
        data = torch.empty(2 * n, dtype=torch.complex128, device=dev)
        op = self.struct()
        N.call("fdfd_assemble_deriv_csr", C.byref(op), code, _ptr(indptr), _ptr(indices), _ptr(data),
               stream_ptr())
        return sp.csr_matrix((data.cpu().numpy(), indices.cpu().numpy(), indptr.cpu().numpy()),
                             shape=(n, n))

    # ---- K2 -----------------------------------------------------------------
    def residual(self, x, b):
        x = as_c128(x)
        b = as_c128(b)
        nrhs = x.numel() // self.n
        r = torch.empty_like(b)
        op = self.struct()
        N.call("fdfd_residual", C.byref(op), _ptr(x), _ptr(b), _ptr(r), nrhs, stream_ptr())
        return r

    def apply(self, x, transpose=False):
        x = as_c128(x)
        nrhs = x.numel() // self.n
        y = torch.empty_like(x)
        op = self.struct()
        N.call("fdfd_apply", C.byref(op), _ptr(x), _ptr(y), nrhs, int(bool(transpose)), stream_ptr())
        return y

    # ---- K8 -----------------------------------------------------------------
    def fields(self, X, averaging=True, eps=None):
        X = as_c128(X).reshape(-1)
        f1 = torch.empty_like(X)
        f2 = torch.empty_like(X)
        op = self.struct(averaging=averaging, eps=eps)
        N.call("fdfd_fields", C.byref(op), _ptr(X), _ptr(f1), _ptr(f2), stream_ptr())
        return f1, f2

    # ---- K9 -----------------------------------------------------------------
    def grad_eps(self, lam, E):
        lam = as_c128(lam).reshape(-1)
        E = as_c128(E).reshape(-1)
        g = torch.empty(self.n, dtype=torch.float64, device=lam.device)
        op = self.struct()
        N.call("fdfd_adjoint_grad_eps", C.byref(op), _ptr(lam), _ptr(E), _ptr(g), stream_ptr())
        return g


def norms(v: torch.Tensor, n: int):
    v = as_c128(v)
    ncol = v.numel() // n
    out = (C.c_double * ncol)()
    N.call("fdfd_norms", _ptr(v), n, ncol, out, stream_ptr())
    return np.array(out[:])


class Symbolic:
    """Nested-dissection front tree of an Nx x Ny periodic grid (host); with
    batch > 1 the forest of `batch` copies (one factorization of `batch`
    operators of that grid)."""

    def __init__(self, Nx, Ny, leaf_area=DEFAULT_LEAF_AREA, batch=1):
        h = C.c_void_p()
        if batch > 1:
            N.call("fdfd_symbolic_create_batch", int(Nx), int(Ny), int(leaf_area), int(batch), C.byref(h))
        else:
            N.call("fdfd_symbolic_create", int(Nx), int(Ny), int(leaf_area), C.byref(h))
        self.handle = h
        self.Nx, self.Ny, self.leaf_area, self.batch = int(Nx), int(Ny), int(leaf_area), int(batch)
        info = N.SymbolicInfo()
        N.call("fdfd_symbolic_info_get", h, C.byref(info))
        self.info = info

    def export(self, which: int, count: int, dtype=np.int32):
        out = np.empty(count, dtype=dtype)
        N.call("fdfd_symbolic_export", self.handle, which, out.ctypes.data_as(C.c_void_p))
        return out

    def __del__(self):
        try:
            if self.handle:
                N.lib().fdfd_symbolic_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


_sym_cache: dict = {}
_sym_lock = threading.Lock()


def symbolic_for(Nx, Ny, leaf_area=DEFAULT_LEAF_AREA, batch=1) -> Symbolic:
    """Symbolic analyses are cached per grid shape and batch size (they
    depend on nothing else)."""
    key = (int(Nx), int(Ny), int(leaf_area)) + ((int(batch),) if batch > 1 else ())
    with _sym_lock:
        s = _sym_cache.get(key)
        if s is None:
            s = Symbolic(*key[:3], batch=int(batch))
            _sym_cache[key] = s
        return s


# Device memory of released factors, kept for the next factor of the same
# grid, precision and right-hand-side count: allocating (and freeing) the
# ~20 GB of a 2048^2 factor costs tens of milliseconds, a quarter of the
# solve itself, so a Simulation created per solve reuses it.  Only factors
# of the process-wide symbolic analyses (symbolic_for, which live as long as
# the process) are kept, at most one per key; release_cached_factors()
# frees them.  Work on a factor is asynchronous (and freeing no longer
# synchronizes the device), so a parked factor carries an event per stream
# it was used on and its next owner's stream waits for them.
_parked = {}
_parked_lock = threading.Lock()


def release_cached_factors():
    """Frees the device memory of released factors kept for reuse."""
    with _parked_lock:
        hs = [h for h, _ in _parked.values()]
        _parked.clear()
    for h in hs:
        N.lib().fdfd_factor_destroy(h)


class Factor:
    """A numeric multifrontal factorization of one operator on the device."""

    def __init__(self, sym: Symbolic, precision="c128", max_nrhs=1, pivot_tol=None, fused_max_m=None):
        if precision not in N.PREC:
            raise ValueError("precision must be 'c128', 'c64' or 'c64tc'")
        device()
        self.sym, self.precision, self.max_nrhs = sym, precision, int(max_nrhs)
        skey = (sym.Nx, sym.Ny, sym.leaf_area) + ((sym.batch,) if sym.batch > 1 else ())
        shared = _sym_cache.get(skey) is sym
        self._key = skey + (precision, self.max_nrhs) if shared else None
        h = None
        self._events = {}
        if self._key is not None:
            with _parked_lock:
                got = _parked.pop(self._key, None)
            if got is not None:
                h, events = got
                cur = torch.cuda.current_stream()
                for ev in events:
                    cur.wait_event(ev)
        if h is None:
            h = C.c_void_p()
            try:
                N.call("fdfd_factor_create", sym.handle, N.PREC[precision], self.max_nrhs, C.byref(h))
            except N.FDFDError as e:
                if e.code != N.FDFD_ERR_OOM:
                    raise
                # parked factors (and torch's cached blocks) are caches: free
                # them and try once more before reporting the shortage
                release_cached_factors()
                torch.cuda.empty_cache()
                h = C.c_void_p()
                N.call("fdfd_factor_create", sym.handle, N.PREC[precision], self.max_nrhs, C.byref(h))
        self.handle = h
        N.call("fdfd_factor_set_pivot_tol", h, -1.0 if pivot_tol is None else float(pivot_tol))
        N.call("fdfd_factor_set_fused_limit", h, -1 if fused_max_m is None else int(fused_max_m))
        N.call("fdfd_factor_set_wait_limit", h, -1)
        N.call("fdfd_factor_set_graphs", h, 1)
        self.op = None

    def set_graphs(self, on=True):
        """Replay the factorization as a CUDA graph (default) or launch it
        directly."""
        N.call("fdfd_factor_set_graphs", self.handle, int(bool(on)))

    def set_wait_limit(self, polls=None):
        """Polls a bounded wait of the cooperative substitutions makes before
        the solve gives up with DeviceTimeout (None: the built-in limits)."""
        N.call("fdfd_factor_set_wait_limit", self.handle, -1 if polls is None else int(polls))

    @staticmethod
    def bytes_needed(sym: Symbolic, precision="c128", max_nrhs=1) -> int:
        b = C.c_int64()
        N.call("fdfd_factor_bytes", sym.handle, N.PREC[precision], int(max_nrhs), C.byref(b))
        return int(b.value)

    def _used(self):
        # an event at the end of the work just queued on the current stream
        st = torch.cuda.current_stream()
        ev = torch.cuda.Event()
        ev.record(st)
        self._events[st.cuda_stream] = ev

    def numeric(self, op: DeviceOperator):
        s = op.struct()
        N.call("fdfd_factor_numeric", self.handle, C.byref(s), stream_ptr())
        self._last = None
        self._used()
        self.op = op
        self._op_struct = s
        return self

    def _chunks(self, b, n):
        """Right-hand sides in column blocks of at most max_nrhs."""
        nrhs = b.numel() // n
        flat = b.reshape(nrhs, n)
        for c0 in range(0, nrhs, self.max_nrhs):
            yield flat[c0:c0 + self.max_nrhs].contiguous()

    def apply_inverse(self, b, transpose=False):
        """One application x = A^-1 b (no refinement), complex128 device."""
        b = as_c128(b)
        n = self.op.n
        outs = []
        for blk in self._chunks(b, n):
            x = torch.empty_like(blk)
            N.call("fdfd_factor_solve", self.handle, _ptr(blk), _ptr(x), blk.shape[0], int(bool(transpose)),
                   stream_ptr())
            outs.append(x)
        self._used()
        return torch.cat(outs).reshape(b.shape)

    def solve(self, b, transpose=False, tol=1e-12, max_iter=10, op: DeviceOperator | None = None,
              raise_on_fail=False, method="ir", restart=20):
        """x with ||b - A x|| <= tol ||b|| per column: FP64 iterative
        refinement (method='ir') or factor-preconditioned GMRES
        (method='gmres', one column at a time)."""
        op = self.op if op is None else op
        b = as_c128(b)
        n = op.n
        s = op.struct()
        outs, worst, iters = [], 0.0, 0
        blocks = self._chunks(b, n) if method == "ir" else (col.contiguous() for col in b.reshape(-1, n))
        for blk in blocks:
            x = torch.empty_like(blk)
            if method == "gmres":
                code = N.lib().fdfd_solve_gmres(self.handle, C.byref(s), _ptr(blk), _ptr(x), int(bool(transpose)),
                                                float(tol), int(max_iter), int(restart), stream_ptr())
            else:
                code = N.lib().fdfd_solve_refined(self.handle, C.byref(s), _ptr(blk), _ptr(x),
                                                  blk.reshape(-1, n).shape[0], int(bool(transpose)), float(tol),
                                                  int(max_iter), stream_ptr())
            if code != N.FDFD_ERR_NOT_CONVERGED or raise_on_fail:
                N.check(code, "fdfd_solve_refined")
            st = self._raw_stats()
            worst, iters = max(worst, st["rel_residual"]), max(iters, st["refine_iters"])
            outs.append(x)
        self._used()
        self._last = (worst, iters)
        return torch.cat(outs).reshape(b.shape)

    def coefficients(self) -> torch.Tensor:
        """The operator coefficients the last numeric factorization stored,
        complex128 (5, n): centre, (i-1, j), (i+1, j), (i, j-1), (i, j+1)
        of cell k = i Ny + j (fdfd_factor_coef_get)."""
        out = torch.empty(5, self.sym.Nx * self.sym.Ny, dtype=torch.complex128,
                          device=device())
        N.call("fdfd_factor_coef_get", self.handle, _ptr(out), stream_ptr())
        return out

    def stats(self) -> dict:
        """Counters of the last factorization and solve (the residual and
        refinement count are the worst over the column blocks of the last
        solve call)."""
        out = self._raw_stats()
        last = getattr(self, "_last", None)
        if last is not None:
            out["rel_residual"], out["refine_iters"] = last
        return out

    def _raw_stats(self) -> dict:
        """The library's counters of the last factorization and of the last
        solve call into it (one column block)."""
        st = N.FactorStats()
        N.call("fdfd_factor_stats_get", self.handle, C.byref(st))
        return {"tiny_pivots": st.tiny_pivots, "refine_iters": st.refine_iters,
                "rel_residual": st.rel_residual, "factor_ms": st.factor_ms, "solve_ms": st.solve_ms,
                "tc_errors": st.tc_errors}

    def __del__(self):
        try:
            h, self.handle = self.handle, None
            if h:
                keep = False
                if self._key is not None:
                    with _parked_lock:
                        keep = self._key not in _parked
                        if keep:
                            _parked[self._key] = (h, list(self._events.values()))
                if not keep:
                    N.lib().fdfd_factor_destroy(h)
        except Exception:
            pass


class BatchFactor(Factor):
    """One forest factorization of `batch` operators of the same grid,
    polarization and frequency (fdfd_factor_numeric_batch): every level's
    launches cover the fronts of all of them."""

    def __init__(self, sym: Symbolic, precision="c64", max_nrhs=8, pivot_tol=None, fused_max_m=None):
        if sym.batch < 2:
            raise ValueError("BatchFactor needs a batch symbolic (symbolic_for(..., batch=B), B >= 2)")
        super().__init__(sym, precision, max_nrhs, pivot_tol, fused_max_m)
        self.batch = sym.batch
        self.ops = None

    def numeric(self, ops):
        if len(ops) != self.batch:
            raise ValueError(f"BatchFactor.numeric: {len(ops)} operators for a batch of {self.batch}")
        structs = (N.Operator * self.batch)(*[o.struct() for o in ops])
        N.call("fdfd_factor_numeric_batch", self.handle, structs, self.batch, stream_ptr())
        self._used()
        self.ops = list(ops)   # their buffers are read by the queued coefficient kernels
        self.op = None
        return self

    def solve_batch(self, rhs, tol=1e-10, max_iter=30, raise_on_fail=False):
        """rhs: list of `batch` device or host arrays (nrhs_b, n) (nrhs_b <= 8;
        None or 0 rows for a problem with nothing to solve).  Returns (list
        of (nrhs_b, n) complex128 device tensors, list of per-problem worst
        relative residuals)."""
        n = self.sym.Nx * self.sym.Ny
        blocks = [None if r is None else as_c128(r).reshape(-1, n) for r in rhs]
        nr = max([b.shape[0] for b in blocks if b is not None] + [1])
        if nr > self.max_nrhs:
            raise ValueError(f"at most {self.max_nrhs} right-hand sides per problem")
        B = torch.zeros((nr, self.batch, n), dtype=torch.complex128, device=device())
        for p, blk in enumerate(blocks):
            if blk is not None and blk.shape[0]:
                B[:blk.shape[0], p] = blk
        X = torch.empty_like(B)
        rel = (C.c_double * (nr * self.batch))()
        code = N.lib().fdfd_solve_refined_batch(self.handle, _ptr(B), _ptr(X), nr, float(tol), int(max_iter), rel,
                                                stream_ptr())
        if code != N.FDFD_ERR_NOT_CONVERGED or raise_on_fail:
            N.check(code, "fdfd_solve_refined_batch")
        self._used()
        rr = np.array(rel[:]).reshape(nr, self.batch)
        xs, worst = [], []
        for p, blk in enumerate(blocks):
            k = 0 if blk is None else blk.shape[0]
            xs.append(X[:k, p].contiguous())
            worst.append(float(rr[:k, p].max()) if k else 0.0)
        return xs, worst


class StencilOperator:
    """An explicit periodic 5-point operator on an Nx x Ny grid (complex128
    coefficients [5][n] on the device); factored by the same engine."""

    def __init__(self, Nx, Ny, stencil: torch.Tensor, pol="Ez"):
        self.Nx, self.Ny, self.pol = int(Nx), int(Ny), pol
        self.stencil = stencil.reshape(5, -1).contiguous()
        assert self.stencil.dtype == torch.complex128 and self.stencil.shape[1] == self.Nx * self.Ny

    @property
    def n(self):
        return self.Nx * self.Ny

    def struct(self, **_):
        op = N.Operator()
        op.Nx, op.Ny, op.pol, op.averaging = self.Nx, self.Ny, N.POL[self.pol], 0
        op.omega, op.L0, op.xlen, op.ylen = 1.0, 1.0, 1.0, 1.0
        op.stencil = self.stencil.data_ptr()
        return op

    def apply(self, x, transpose=False):
        x = as_c128(x)
        y = torch.empty_like(x)
        op = self.struct()
        N.call("fdfd_apply", C.byref(op), _ptr(x), _ptr(y), x.numel() // self.n, int(bool(transpose)),
               stream_ptr())
        return y

    @staticmethod
    def mode_slice(pol, eps_slice, omega, dl, L0, shift, average):
        """Slice operator of insert_mode minus shift * I (N x 1 grid)."""
        e = as_f64(eps_slice).reshape(-1)
        Ns = e.numel()
        st = torch.empty(5 * Ns, dtype=torch.complex128, device=e.device)
        N.call("fdfd_mode_stencil", Ns, N.POL[pol], int(bool(average)), _ptr(e), float(omega), float(dl),
               float(L0), float(shift), _ptr(st), stream_ptr())
        return StencilOperator(Ns, 1, st, pol)


def shift_invert_eigs(op_shifted: StencilOperator, shift: float, k: int, tol=1e-12, max_iter=500,
                      seed=0):
    """The k eigenpairs of A nearest `shift`, from the factor of A - shift I
    (shift-invert block subspace iteration + Rayleigh-Ritz).  Returns
    (values, vectors (n, k)) ordered by distance to the shift, vectors of
    unit 2-norm.  Replaces ARPACK's eigs(A, k, sigma=shift, which='LM')
    (fdfdpy/linalg.py:110-119)."""
    n = op_shifted.n
    kb = int(min(n, max(k + 2, 2), 8))
    fac = Factor(symbolic_for(op_shifted.Nx, op_shifted.Ny, 1), "c128", max_nrhs=kb).numeric(op_shifted)
    g = torch.Generator(device="cpu").manual_seed(seed)
    V = torch.randn(n, kb, generator=g, dtype=torch.float64).to(torch.complex128).to(device())
    V, _ = torch.linalg.qr(V)
    lam = vecs = None
    for _ in range(max_iter):
        W = fac.apply_inverse(V.T.contiguous()).reshape(kb, n).T
        V, _ = torch.linalg.qr(W)
        AV = op_shifted.apply(V.T.contiguous()).reshape(kb, n).T
        H = (V.conj().T @ AV).cpu()
        mu, S = torch.linalg.eig(H)
        order = torch.argsort(mu.abs())
        mu, S = mu[order], S[:, order]
        Y = V @ S.to(V.device)
        R = op_shifted.apply(Y.T.contiguous()).reshape(kb, n).T - Y * mu.to(V.device)[None, :]
        res = torch.linalg.vector_norm(R[:, :k], dim=0) / torch.clamp(mu[:k].abs().to(V.device), min=1e-300)
        lam = (mu[:k] + shift).numpy()
        vecs = Y[:, :k]
        V, _ = torch.linalg.qr(Y)
        if float(torch.max(torch.linalg.vector_norm(R[:, :k], dim=0))) <= tol * max(1.0, float(
                torch.max(mu.abs()))) or float(res.max()) <= tol:
            break
    vecs = vecs / torch.linalg.vector_norm(vecs, dim=0, keepdim=True)
    return lam, vecs
