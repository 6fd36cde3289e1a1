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
