"""Continuous-batching solve server on one GPU (no counterpart in the
reference; it serves the same solves as solver_direct,
fdfdpy/linalg.py:122-149, for many independent requests).

* Requests (eps_r, omega, dl, NPML, pol, right-hand sides) arrive over time
  and wait in an admission queue.
* Requests that have arrived, miss the factor cache and share a grid,
  polarization and frequency are factored together: up to `batch_max` of
  them form one forest factorization (engine.BatchFactor,
  fdfd_factor_numeric_batch), so every level's front updates of all of
  them run in one launch, and their right-hand sides are refined together
  (fdfd_solve_refined_batch).  The batch size of each grid comes from the
  project's autotuner (fdfdpy_gb300.autotune) when `autotune` is set.
* A request (or batch) is admitted into a free slot when the device memory
  its factor needs (fdfd_factor_bytes of its symbolic) fits in the budget
  next to what is resident.  Each slot is one CUDA stream driven by a
  worker thread; the engine's C calls release the GIL, so the kernels of
  different slots overlap on the device.
* Factors stay resident in an LRU cache (one entry per factorization; each
  member operator, keyed by a hash of eps_r and the scalars, points at its
  entry and its place in the batch); a request whose operator is cached
  skips the factorization and only solves (its right-hand sides are new).
  An entry is used by one slot at a time (its solve workspace is per
  factor).
* Every result is the complex64 (or complex128) factor refined in FP64 to
  the requested residual; a request whose refinement stalls is solved again
  with a complex128 factor.  Each result states its residual.  Latency is
  completion minus arrival; the server reports p50/p99 and solves/s (one
  solve = one right-hand side).
"""
from __future__ import annotations

import hashlib
import itertools
import threading
import time
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np
import torch

from . import engine


@dataclass(eq=False)  # a request is equal only to itself (the queue looks requests up by identity)
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
    batch: int = 1                # problems factored together with this one
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
    def family(self):
        """Requests of one family may share a batch factorization (same grid,
        polarization and frequency: one scaling suits them all)."""
        return (tuple(self.eps_r.shape), self.pol, float(self.omega), float(self.dl),
                tuple(int(v) for v in self.NPML), float(self.L0))

    @property
    def nrhs(self):
        return self.rhs.shape[0]


@dataclass
class _CacheEntry:
    ops: list
    fac: object
    bytes: int
    keys: list
    lock: threading.Lock = field(default_factory=threading.Lock)
    users: int = 0


class SolveServer:
    """Run a list of timed requests; see the module docstring."""

    def __init__(self, slots=4, precision="c64", tol=1e-10, max_iter=40, memory_budget=None,
                 cache_budget=None, leaf_area=None, batch_max=4, autotune=None):
        engine.device()
        self.slots, self.precision, self.tol, self.max_iter = int(slots), precision, tol, max_iter
        free, total = torch.cuda.mem_get_info()
        self.budget = int(memory_budget if memory_budget is not None else 0.8 * free)
        self.cache_budget = int(cache_budget if cache_budget is not None else 0.5 * self.budget)
        self.cache: OrderedDict[int, _CacheEntry] = OrderedDict()   # entry id -> entry (LRU order)
        self.key_index: dict = {}                                   # operator key -> (entry id, position)
        self._ids = itertools.count()
        self.resident = 0          # bytes of cached + in-use factors
        self.cv = threading.Condition()
        self.leaf_area = leaf_area
        self.batch_max = max(1, int(batch_max))
        self.autotune = autotune
        self.factorizations = 0

    # ---- memory accounting ---------------------------------------------------
    def _sym(self, shape, batch=1):
        leaf = engine.DEFAULT_LEAF_AREA if self.leaf_area is None else self.leaf_area
        return engine.symbolic_for(shape[0], shape[1], leaf, batch)

    def _need(self, shape, batch=1):
        return engine.Factor.bytes_needed(self._sym(shape, batch), self.precision, 8)

    def _fused(self, shape):
        return None if self.autotune is None else self.autotune.fused_for(shape, self.precision)

    def _batch_limit(self, shape):
        if self.autotune is not None:
            return max(1, min(self.batch_max, self.autotune.batch_for(shape, self.precision)))
        return self.batch_max

    def _evict_for(self, need):
        """Drop idle cached factors (LRU) until `need` fits (cv held)."""
        for eid in list(self.cache.keys()):
            if self.resident + need <= self.budget:
                break
            ent = self.cache[eid]
            if ent.users == 0:
                del self.cache[eid]
                for k in ent.keys:
                    if self.key_index.get(k, (None,))[0] == eid:
                        del self.key_index[k]
                self.resident -= ent.bytes
        return self.resident + need <= self.budget

    # ---- one unit of work (a cache hit or a batch of misses) on one stream -----
    def _serve(self, reqs, stream, t0, pinned, need=0):
        start = time.perf_counter() - t0
        for r in reqs:
            r.start = start
        ent = eid = None
        try:
            with torch.cuda.stream(stream):
                if pinned is not None:
                    eid, pos = pinned
                    ent = self.cache[eid]
                    reqs[0].cache_hit = True
                    positions = [pos]
                else:
                    ops = [engine.DeviceOperator(r.omega, r.eps_r, r.eps_r.shape[0] * r.dl,
                                                 r.eps_r.shape[1] * r.dl, r.NPML, r.pol, r.L0) for r in reqs]
                    B = len(reqs)
                    shape = reqs[0].eps_r.shape
                    if B > 1:
                        fac = engine.BatchFactor(self._sym(shape, B), self.precision, max_nrhs=8,
                                                 fused_max_m=self._fused(shape))
                        fac.numeric(ops)
                    else:
                        fac = engine.Factor(self._sym(shape), self.precision, max_nrhs=8,
                                            fused_max_m=self._fused(shape)).numeric(ops[0])
                    with self.cv:
                        self.factorizations += 1
                    eid = next(self._ids)
                    ent = _CacheEntry(ops, fac, need, [r.key for r in reqs], users=1)
                    positions = list(range(B))
                ent.lock.acquire()
                try:
                    self._solve_on(ent, reqs, positions)
                finally:
                    # work queued on this stream may still use the factor's solve
                    # workspace: it must finish before another stream takes the factor
                    try:
                        stream.synchronize()
                    finally:
                        ent.lock.release()
        except Exception as e:  # e.g. the factor did not fit: these requests fail, the slot goes on
            for r in reqs:
                if r.error is None and r.x is None:
                    r.error = repr(e)
        with self.cv:
            if ent is None:
                self.resident -= need          # nothing was built
            else:
                ent.users -= 1
                if pinned is not None:
                    pass                       # a cache hit: stays resident
                elif ent.bytes <= self.cache_budget:
                    self.cache[eid] = ent      # keep it resident for reuse
                    for p, k in enumerate(ent.keys):
                        self.key_index.setdefault(k, (eid, p))
                else:
                    self.resident -= ent.bytes  # not kept: its memory is released
                    ent = None
            self.cv.notify_all()
        done = time.perf_counter() - t0
        for r in reqs:
            r.done = done

    def _solve_on(self, ent, reqs, positions):
        fac = ent.fac
        try:
            if isinstance(fac, engine.BatchFactor):
                rhs = [None] * fac.batch
                for r, p in zip(reqs, positions):
                    rhs[p] = torch.from_numpy(r.rhs).to(engine.device(), non_blocking=True)
                xs, worst = fac.solve_batch(rhs, tol=self.tol, max_iter=self.max_iter)
                iters = fac.stats()["refine_iters"]
                out = [(xs[p], worst[p], iters) for p in positions]
            else:
                b = torch.from_numpy(reqs[0].rhs).to(engine.device(), non_blocking=True)
                x = fac.solve(b, tol=self.tol, max_iter=self.max_iter, op=ent.ops[0])
                st = fac.stats()
                out = [(x, st["rel_residual"], st["refine_iters"])]
        except Exception as e:  # reported per request, the server keeps going
            for r in reqs:
                r.error = repr(e)
            return
        for r, p, (x, rel, iters) in zip(reqs, positions, out):
            r.batch = len(ent.keys)
            try:
                if not rel <= self.tol and self.precision != "c128":
                    # a nearly singular operator (a resonance of this eps) can leave the
                    # complex64 factor too inaccurate for the refinement to contract:
                    # solve this request again with a complex128 factor
                    op = ent.ops[p]
                    fac128 = engine.Factor(self._sym(r.eps_r.shape), "c128", max_nrhs=8).numeric(op)
                    b = torch.from_numpy(r.rhs).to(engine.device())
                    x = fac128.solve(b, tol=self.tol, max_iter=self.max_iter, op=op)
                    st = fac128.stats()
                    rel, iters = st["rel_residual"], st["refine_iters"]
                    r.fallback = True
                    del fac128
                r.x = x.cpu().numpy()
                r.rel_residual, r.refine_iters = rel, iters
            except Exception as e:
                r.error = repr(e)

    def _take_batch(self, pending, idx, now, realtime, taken):
        """The request at idx plus up to batch_limit - 1 later ones that have
        arrived, miss the cache, are not already queued in this batch and
        share its family (cv held)."""
        first = pending[idx]
        group = [first]
        keys = {first.key}
        limit = self._batch_limit(first.eps_r.shape)
        j = idx + 1
        while len(group) < limit and j < len(pending) and j < idx + 256:
            r = pending[j]
            if realtime and r.arrival > now:
                break
            if (j not in taken and r.family == first.family and r.key not in keys
                    and r.key not in self.key_index):
                group.append(r)
                keys.add(r.key)
                taken.add(j)
            j += 1
        return group

    def run(self, requests, realtime=True):
        """Serve `requests` (sorted by arrival).  Returns summary metrics."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        if self.autotune is not None:
            # tune every grid of the stream before the clock starts (timing
            # inside the loop would compete with the slots' work)
            for shape in sorted({tuple(r.eps_r.shape) for r in reqs}):
                self.autotune.config_for(shape, self.precision)
        pending = list(reqs)
        streams = [torch.cuda.Stream() for _ in range(self.slots)]
        free_slots = list(range(self.slots))
        threads = []
        taken = set()             # indices already served as part of an earlier batch
        t0 = time.perf_counter()
        idx = 0
        while idx < len(pending) or threads:
            now = time.perf_counter() - t0
            with self.cv:
                threads = [t for t in threads if t[0].is_alive() or not self._reap(t, free_slots)]
                while idx < len(pending) and free_slots and (not realtime or pending[idx].arrival <= now):
                    if idx in taken:
                        idx += 1
                        continue
                    req = pending[idx]
                    hit = self.key_index.get(req.key)
                    if hit is not None and hit[0] in self.cache:     # pin the cached factor
                        ent = self.cache[hit[0]]
                        ent.users += 1
                        self.cache.move_to_end(hit[0])
                        group, pinned, need = [req], hit, 0
                    else:
                        group = self._take_batch(pending, idx, now, realtime, taken)
                        pinned = None
                        need = self._need(req.eps_r.shape, len(group))
                        while len(group) > 1 and need > self.budget:
                            taken.discard(pending.index(group.pop()))
                            need = self._need(req.eps_r.shape, len(group))
                    if need and not self._evict_for(need):
                        if not threads:
                            for r in group:
                                r.error = "request needs more memory than the budget"
                                r.done = r.start = now
                            idx += 1
                            continue
                        for r in group[1:]:
                            taken.discard(pending.index(r))
                        break
                    self.resident += need
                    slot = free_slots.pop()
                    th = threading.Thread(target=self._serve, args=(group, streams[slot], t0, pinned, need),
                                          daemon=True)
                    th.start()
                    threads.append((th, slot))
                    idx += 1
                if threads or idx < len(pending):
                    self.cv.wait(timeout=0.002)
        makespan = time.perf_counter() - t0
        return self.summary(reqs, makespan, self.factorizations)

    @staticmethod
    def _reap(t, free_slots):
        t[0].join()
        free_slots.append(t[1])
        return True

    @staticmethod
    def summary(reqs, makespan, factorizations=None):
        ok = [r for r in reqs if r.error is None]
        lat = np.array([r.done - r.arrival for r in ok]) if ok else np.array([np.nan])
        solves = sum(r.nrhs for r in ok)
        return {
            "requests": len(reqs), "failed": len(reqs) - len(ok), "solves": solves,
            "makespan_s": makespan, "solves_per_s": solves / makespan if makespan > 0 else float("nan"),
            "requests_per_s": len(ok) / makespan if makespan > 0 else float("nan"),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "cache_hits": sum(r.cache_hit for r in ok),
            "factorizations": factorizations,
            "batched_requests": sum(r.batch > 1 and not r.cache_hit for r in ok),
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
