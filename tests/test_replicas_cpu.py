"""Replica aggregation over 2 gloo ranks on the CPU, and the serving
workload generator (host logic, no GPU)."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from fdfdpy_gb300.replicas import max_over_ranks, barrier
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier()
    v = max_over_ranks(10.0 + rank)
    q.put((rank, v))
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 11.0), (1, 11.0)]


def test_single_process_is_identity():
    from fdfdpy_gb300.replicas import max_over_ranks
    assert max_over_ranks(3.5) == 3.5


def test_serving_stream_distribution():
    from fdfdpy_gb300.serving import make_stream
    reqs = make_stream(n_requests=512, rate=20.0, seed=0, sides=(16, 24, 32, 40, 48), block=2)
    assert len(reqs) == 512
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0) and 15 < 512 / arr[-1] < 26      # Poisson, rate 20/s
    sides = np.array([r.eps_r.shape[0] for r in reqs])
    assert set(sides) <= {16, 24, 32, 40, 48}
    nrhs = np.array([r.nrhs for r in reqs])
    assert nrhs.min() >= 1 and nrhs.max() <= 8
    pols = np.array([r.pol == "Ez" for r in reqs])
    assert 0.35 < pols.mean() < 0.65
    keys = [r.key for r in reqs]
    repeats = len(keys) - len(set(keys))
    assert 0.15 < repeats / 512 < 0.35                                  # ~25% reuse an eps
    r0 = reqs[0]
    assert r0.rhs.shape == (r0.nrhs, r0.eps_r.size) and r0.rhs.dtype == np.complex128
