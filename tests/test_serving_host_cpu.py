"""Host logic of the solve server on the CPU: batching of cache misses by
family, LRU eviction of idle factors, and admission by memory in the
dispatch loop.  The device work of one served unit (a batch factorization
and its refinement on a slot's stream) is replaced by a fake that only
returns the unit's memory, so the dispatcher runs as it does on a GPU."""
import time
import types

import numpy as np
import pytest
import torch

from fdfdpy_gb300 import serving
from fdfdpy_gb300.serving import Request, SolveServer, _CacheEntry


@pytest.fixture
def make_server(monkeypatch):
    monkeypatch.setattr(serving.engine, "device", lambda: torch.device("cpu"))
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda *a: (1 << 30, 1 << 30))

    def make(budget, batch_max=4, slots=2):
        return SolveServer(slots=slots, memory_budget=budget, batch_max=batch_max)
    return make


def _req(seed, shape=(8, 8), pol="Ez", omega=1.0, arrival=0.0, nrhs=1):
    rng = np.random.default_rng(seed)
    return Request(eps_r=1 + rng.random(shape), rhs=np.zeros((nrhs, shape[0] * shape[1]), complex), omega=omega,
                   dl=0.02, NPML=(2, 2), pol=pol, arrival=arrival, rid=seed)


def test_take_batch_groups_arrived_misses_of_one_family(make_server):
    s = make_server(budget=1 << 20, batch_max=3)
    a, b, c = _req(1), _req(2, pol="Hz"), _req(3)
    d = _req(1)                      # the same operator as a
    e, f = _req(5), _req(6, arrival=5.0)
    pending = [a, b, c, d, e, f]
    taken = set()
    group = s._take_batch(pending, 0, now=1.0, realtime=True, taken=taken)
    assert group == [a, c, e]        # b: other family; d: a's operator again; limit 3
    assert taken == {2, 4}
    # a cached operator is not factored again; a request that has not arrived ends the scan
    s.key_index[c.key] = (0, 0)
    taken = set()
    assert s._take_batch(pending, 0, now=1.0, realtime=True, taken=taken) == [a, e]
    assert taken == {4}
    assert s._take_batch([a, f, e], 0, now=1.0, realtime=True, taken=set()) == [a]


def test_evict_for_drops_idle_entries_in_lru_order(make_server):
    s = make_server(budget=350)
    for eid, users in ((0, 0), (1, 1), (2, 0)):
        s.cache[eid] = _CacheEntry(ops=[], fac=None, bytes=100, keys=[f"k{eid}"], users=users)
        s.key_index[f"k{eid}"] = (eid, 0)
    s.resident = 300
    assert s._evict_for(100)                       # entry 0 (idle, least recent) goes
    assert list(s.cache) == [1, 2] and "k0" not in s.key_index and s.resident == 200
    assert not s._evict_for(300)                   # entry 1 is in use: only entry 2 can go
    assert list(s.cache) == [1] and s.resident == 100


def test_dispatch_admits_by_memory_and_serves_every_request(make_server, monkeypatch):
    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: None)
    s = make_server(budget=250, batch_max=4, slots=2)
    s._need = lambda shape, batch=1: (10_000 if shape[0] == 16 else 100) * batch
    peak = {"resident": 0, "batch": 0}

    def fake_serve(self, reqs, stream, t0, pinned, need=0):
        with self.cv:
            peak["resident"] = max(peak["resident"], self.resident)
            peak["batch"] = max(peak["batch"], len(reqs))
        time.sleep(0.01)
        with self.cv:
            for r in reqs:
                r.done = time.perf_counter() - t0
                r.batch = len(reqs)
                r.rel_residual = 0.0
            self.factorizations += 1
            self.resident -= need
            self.cv.notify_all()

    s._serve = types.MethodType(fake_serve, s)
    reqs = [_req(i, pol="Ez" if i % 3 else "Hz") for i in range(12)] + [_req(99, shape=(16, 16))]
    out = s.run(reqs, realtime=False)
    big = reqs[-1]
    assert big.error == "request needs more memory than the budget"
    assert all(r.error is None for r in reqs[:-1]) and all(r.done > 0 for r in reqs[:-1])
    assert out["failed"] == 1 and out["requests"] == 13
    assert peak["batch"] == 2            # a batch of 4 (400 bytes) does not fit 250: cut to 2
    assert peak["resident"] <= s.budget
    assert s.resident == 0               # every unit gave its memory back


class _Stream:
    def synchronize(self):
        pass


class _FakeEngine:
    """Factor / BatchFactor / DeviceOperator stand-ins that solve nothing:
    x = b, a residual chosen per operator, and a factorization that fails
    for 12 x 12 grids."""

    def __init__(self, bad_residual_keys):
        eng = self

        class DeviceOperator:
            def __init__(self, omega, eps_r, xlen, ylen, NPML, pol, L0):
                self.eps_r = eps_r

        class Factor:
            def __init__(self, sym, precision, max_nrhs=8, fused_max_m=None):
                self.precision = precision

            def numeric(self, op):
                if op.eps_r.shape == (12, 12):
                    raise RuntimeError("factor_create: device allocation failed")
                self.op = op
                return self

            def solve(self, b, tol, max_iter, op=None):
                bad = self.precision != "c128" and eng.key(op.eps_r) in bad_residual_keys
                self._st = {"rel_residual": 1e-3 if bad else 1e-12, "refine_iters": 3}
                return b.clone()

            def stats(self):
                return self._st

        class BatchFactor:
            def __init__(self, sym, precision, max_nrhs=8, fused_max_m=None):
                self.batch = sym[2]

            def numeric(self, ops):
                self.ops = ops
                return self

            def solve_batch(self, rhs, tol, max_iter):
                return [b.clone() for b in rhs], [1e-12] * len(rhs)

            def stats(self):
                return {"refine_iters": 2}

        self.DeviceOperator, self.Factor, self.BatchFactor = DeviceOperator, Factor, BatchFactor

    @staticmethod
    def key(eps):
        return eps.tobytes()


def test_serve_caches_reuses_falls_back_and_accounts_memory(make_server, monkeypatch):
    """The real per-unit path (_serve / _solve_on) over fake engine objects,
    one slot: a repeated operator is a cache hit on the entry its first
    request built, a request whose complex64 refinement stalls is solved
    again in complex128, a factorization that fails fails its requests only,
    and the resident bytes are exactly those of the cached entries."""
    reqs = [_req(1), _req(2), _req(1), _req(3, shape=(12, 12)), _req(4), _req(4, nrhs=3)]
    fake = _FakeEngine({_FakeEngine.key(reqs[4].eps_r)})
    monkeypatch.setattr(serving.engine, "DeviceOperator", fake.DeviceOperator)
    monkeypatch.setattr(serving.engine, "Factor", fake.Factor)
    monkeypatch.setattr(serving.engine, "BatchFactor", fake.BatchFactor)
    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: _Stream())
    monkeypatch.setattr(torch.cuda, "stream", lambda s: __import__("contextlib").nullcontext())
    s = make_server(budget=10_000, batch_max=1, slots=1)
    s._sym = lambda shape, batch=1: (shape[0], shape[1], batch)
    s._need = lambda shape, batch=1: 100 * batch
    out = s.run(reqs, realtime=False)
    assert reqs[3].error is not None and "device allocation failed" in reqs[3].error
    ok = [r for i, r in enumerate(reqs) if i != 3]
    assert all(r.error is None and r.x is not None for r in ok)
    assert [r.cache_hit for r in reqs] == [False, False, True, False, False, True]
    assert np.array_equal(reqs[5].x, reqs[5].rhs)            # x = b from the fake factor
    assert reqs[4].fallback and reqs[5].fallback and not reqs[0].fallback
    assert out["factorizations"] == 3 and out["failed"] == 1 and out["cache_hits"] == 2
    assert s.resident == sum(e.bytes for e in s.cache.values()) == 300
    assert all(e.users == 0 for e in s.cache.values())
