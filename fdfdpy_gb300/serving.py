"""Continuous-batching solve server on one GPU (no counterpart in the
reference; it serves the same solves as solver_direct,
fdfdpy/linalg.py:122-149, for many independent requests).

* Requests (eps_r, omega, dl, NPML, pol, right-hand sides) arrive over time
  and wait in an admission queue.
* A request is admitted into a free slot when the device memory it needs
  (its factor, from the symbolic analysis: fdfd_factor_bytes) fits in the
  budget next to what is resident.  Each slot is one CUDA stream driven by
  a worker thread; the engine's C calls release the GIL, so the kernels of
  different requests overlap on the device.
* Factors stay resident in an LRU cache keyed by the operator (a hash of
  eps_r and the scalars); a request whose operator is cached skips the
  factorization and only solves (its right-hand sides are new).  A factor
  is used by one request at a time (its solve workspace is per factor).
* Every result is the complex64 (or complex128) factor refined in FP64 to
  the requested residual; each result states its residual.  Latency is
  completion minus arrival; the server reports p50/p99 and solves/s (one
  solve = one right-hand side).
"""
from __future__ import annotations

import hashlib
import threading
import time
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np
import torch

from . import engine


@dataclass
class Request:
    eps_r: np.ndarray
    rhs: np.ndarray               # (nrhs, Nx*Ny) complex128 right-hand sides b
    omega: float
    dl: float
    NPML: tuple
    pol: str
    L0: float = 1e-6
    arrival: float = 0.0          # seconds after the server start
    rid: int = 0
    # filled in by the server
    x: np.ndarray | None = None
    start: float = 0.0
    done: float = 0.0
    cache_hit: bool = False
    rel_residual: float = float("nan")
    refine_iters: int = 0
    fallback: bool = False        # solved again with a complex128 factor
    error: str | None = None

    @property
    def key(self):
        k = self.__dict__.get("_key")
        if k is None:
            h = hashlib.blake2b(np.ascontiguousarray(self.eps_r, dtype=np.float64).tobytes(), digest_size=16)
            h.update(repr((self.eps_r.shape, float(self.omega), float(self.dl),
                           tuple(int(v) for v in self.NPML), self.pol, float(self.L0))).encode())
            k = self.__dict__["_key"] = h.hexdigest()
        return k

    @property
    def nrhs(self):
        return self.rhs.shape[0]


@dataclass
class _CacheEntry:
    op: object
    fac: object
    bytes: int
    lock: threading.Lock = field(default_factory=threading.Lock)
    users: int = 0


class SolveServer:
    """Run a list of timed requests; see the module docstring."""

    def __init__(self, slots=4, precision="c64", tol=1e-10, max_iter=40, memory_budget=None,
                 cache_budget=None, leaf_area=None):
        engine.device()
        self.slots, self.precision, self.tol, self.max_iter = int(slots), precision, tol, max_iter
        free, total = torch.cuda.mem_get_info()
        self.budget = int(memory_budget if memory_budget is not None else 0.8 * free)
        self.cache_budget = int(cache_budget if cache_budget is not None else 0.5 * self.budget)
        self.cache: OrderedDict[str, _CacheEntry] = OrderedDict()
        self.resident = 0          # bytes of cached + in-use factors
        self.cv = threading.Condition()
        self.leaf_area = leaf_area

    # ---- memory accounting ---------------------------------------------------
    def _need(self, req):
        sym = engine.symbolic_for(*req.eps_r.shape) if self.leaf_area is None else \
            engine.symbolic_for(*req.eps_r.shape, self.leaf_area)
        return engine.Factor.bytes_needed(sym, self.precision, 8), sym

    def _evict_for(self, need):
        """Drop idle cached factors (LRU) until `need` fits (cv held)."""
        for k in list(self.cache.keys()):
            if self.resident + need <= self.budget:
                break
            ent = self.cache[k]
            if ent.users == 0:
                del self.cache[k]
                self.resident -= ent.bytes
        return self.resident + need <= self.budget

    # ---- one request on one stream ---------------------------------------------
    def _serve(self, req, stream, t0):
        req.start = time.perf_counter() - t0
        key = req.key
        with torch.cuda.stream(stream):
            ent = req.__dict__.pop("_pinned", None)   # cache hit pinned at admission
            if ent is not None:
                req.cache_hit = True
                ent.lock.acquire()
                fac, op = ent.fac, ent.op
            else:
                need, sym = self._need(req)
                op = engine.DeviceOperator(req.omega, req.eps_r, req.eps_r.shape[0] * req.dl,
                                           req.eps_r.shape[1] * req.dl, req.NPML, req.pol, req.L0)
                fac = engine.Factor(sym, self.precision, max_nrhs=8).numeric(op)
                ent = _CacheEntry(op, fac, need, users=1)
                ent.lock.acquire()
            try:
                b = torch.from_numpy(req.rhs).to(engine.device(), non_blocking=True)
                x = fac.solve(b, tol=self.tol, max_iter=self.max_iter, op=op)
                st = fac.stats()
                if not st["rel_residual"] <= self.tol and self.precision != "c128":
                    # a nearly singular operator (a resonance of this eps) can leave the
                    # complex64 factor too inaccurate for the refinement to contract:
                    # solve this request again with a complex128 factor
                    fac128 = engine.Factor(fac.sym, "c128", max_nrhs=fac.max_nrhs).numeric(op)
                    x = fac128.solve(b, tol=self.tol, max_iter=self.max_iter, op=op)
                    st = fac128.stats()
                    req.fallback = True
                    del fac128
                req.x = x.cpu().numpy()
                req.rel_residual, req.refine_iters = st["rel_residual"], st["refine_iters"]
            except Exception as e:  # reported per request, the server keeps going
                req.error = repr(e)
            finally:
                # work queued on this stream may still use the factor's solve
                # workspace: it must finish before another stream takes the factor
                try:
                    stream.synchronize()
                finally:
                    ent.lock.release()
        with self.cv:
            ent.users -= 1
            if self.cache.get(key) is ent:
                pass                           # a cache hit: stays resident
            elif key not in self.cache and ent.bytes <= self.cache_budget:
                self.cache[key] = ent          # keep it resident for reuse
            else:
                self.resident -= ent.bytes     # not kept: its memory is released
                del ent
            self.cv.notify_all()
        req.done = time.perf_counter() - t0

    def run(self, requests, realtime=True):
        """Serve `requests` (sorted by arrival).  Returns summary metrics."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending = list(reqs)
        streams = [torch.cuda.Stream() for _ in range(self.slots)]
        free_slots = list(range(self.slots))
        threads = []
        t0 = time.perf_counter()
        idx = 0
        while idx < len(pending) or threads:
            now = time.perf_counter() - t0
            with self.cv:
                threads = [t for t in threads if t[0].is_alive() or not self._reap(t, free_slots)]
                while idx < len(pending) and free_slots and (not realtime or pending[idx].arrival <= now):
                    req = pending[idx]
                    hit = self.cache.get(req.key)
                    if hit is not None:          # pin the cached factor for this request
                        hit.users += 1
                        self.cache.move_to_end(req.key)
                        req.__dict__["_pinned"] = hit
                    need = 0 if hit is not None else self._need(req)[0]
                    if need and not self._evict_for(need):
                        if not threads:
                            req.error = "request needs more memory than the budget"
                            req.done = req.start = now
                            idx += 1
                            continue
                        break
                    self.resident += need
                    slot = free_slots.pop()
                    th = threading.Thread(target=self._serve, args=(req, streams[slot], t0), daemon=True)
                    th.start()
                    threads.append((th, slot))
                    idx += 1
                if threads or idx < len(pending):
                    self.cv.wait(timeout=0.002)
        makespan = time.perf_counter() - t0
        return self.summary(reqs, makespan)

    @staticmethod
    def _reap(t, free_slots):
        t[0].join()
        free_slots.append(t[1])
        return True

    @staticmethod
    def summary(reqs, makespan):
        ok = [r for r in reqs if r.error is None]
        lat = np.array([r.done - r.arrival for r in ok]) if ok else np.array([np.nan])
        solves = sum(r.nrhs for r in ok)
        return {
            "requests": len(reqs), "failed": len(reqs) - len(ok), "solves": solves,
            "makespan_s": makespan, "solves_per_s": solves / makespan if makespan > 0 else float("nan"),
            "requests_per_s": len(ok) / makespan if makespan > 0 else float("nan"),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "cache_hits": sum(r.cache_hit for r in ok),
            "c128_fallbacks": sum(r.fallback for r in ok),
            "max_rel_residual": float(max((r.rel_residual for r in ok), default=float("nan"))),
        }


def make_stream(n_requests=512, rate=20.0, sides=(128, 256, 512, 768, 1024), reuse=0.25, block=8,
                npml=(10, 10), seed=0, omega=None, dl=0.02):
    """The serving workload: Poisson arrivals at `rate` per second, square
    grids with a side drawn uniformly from `sides`, Ez/Hz 50/50, 1-8
    complex Gaussian right-hand sides, eps_r in block x block cells drawn
    from {1, 12.25}; a fraction `reuse` repeats an earlier eps_r (same
    operator) with new right-hand sides."""
    from .constants import C_0
    rng = np.random.default_rng(seed)
    om = 2 * np.pi * C_0 / 1.55e-6 if omega is None else omega
    t = 0.0
    out, history = [], []
    for rid in range(n_requests):
        t += rng.exponential(1.0 / rate)
        if history and rng.random() < reuse:
            eps, pol = history[rng.integers(len(history))]
        else:
            N = int(rng.choice(sides))
            eps = np.kron(rng.choice([1.0, 12.25], size=(N // block, N // block)), np.ones((block, block)))
            pol = "Ez" if rng.random() < 0.5 else "Hz"
            history.append((eps, pol))
        N = eps.shape[0]
        nrhs = int(rng.integers(1, 9))
        rhs = (rng.standard_normal((nrhs, N * N)) + 1j * rng.standard_normal((nrhs, N * N)))
        out.append(Request(eps_r=eps, rhs=rhs, omega=om, dl=dl, NPML=npml, pol=pol, arrival=t, rid=rid))
    return out
