"""The continuous-batching solve server: each result is the same alone and
in the mix (bitwise without batch factorizations -- every request's
arithmetic is then independent of the others' -- and within the mixed-
precision field bar, 1e-8 relative, when requests of one grid share a
forest factorization), cached factors are reused, admission respects the
memory budget, and every result meets its residual tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from fdfdpy_gb300.serving import make_stream
    reqs = make_stream(n_requests=10, rate=1e6, sides=(64, 96, 128, 160), reuse=0.3, seed=5, npml=(8, 8))
    for r in reqs:
        r.arrival = 0.0
    return reqs


def test_alone_equals_mix_and_meets_tolerance():
    from fdfdpy_gb300.serving import SolveServer
    alone = {}
    for r in _requests():
        srv = SolveServer(slots=1, precision="c64", tol=1e-10)
        s = srv.run([r], realtime=False)
        assert s["failed"] == 0
        alone[r.rid] = r.x
    for batch_max, bar in ((1, 1e-12), (4, 1e-8)):
        mix = _requests()
        srv = SolveServer(slots=4, precision="c64", tol=1e-10, batch_max=batch_max)
        s = srv.run(mix, realtime=False)
        assert s["failed"] == 0, [r.error for r in mix if r.error]
        assert s["solves"] == sum(r.nrhs for r in mix)
        assert s["max_rel_residual"] <= 1e-10
        if batch_max > 1:
            assert s["batched_requests"] > 0 and s["factorizations"] < len(mix) - s["cache_hits"]
        for r in mix:
            a = alone[r.rid]
            assert np.linalg.norm(r.x - a) <= bar * np.linalg.norm(a), (batch_max, r.rid)


def test_results_match_oracle():
    from oracle import fdfd_oracle as O
    from fdfdpy_gb300.serving import SolveServer
    reqs = _requests()[:4]
    SolveServer(slots=2, precision="c64", tol=1e-10).run(reqs, realtime=False)
    for r in reqs:
        N = r.eps_r.shape[0]
        A = O.construct_A(r.omega, N * r.dl, N * r.dl, r.eps_r, list(r.NPML), r.pol, r.L0)
        for k in range(r.nrhs):
            assert np.linalg.norm(A @ r.x[k] - r.rhs[k]) <= 1e-10 * np.linalg.norm(r.rhs[k]) * 1.01


def test_admission_budget_and_oversize_request():
    from fdfdpy_gb300 import engine
    from fdfdpy_gb300.serving import SolveServer
    reqs = _requests()[:5]
    need = max(engine.Factor.bytes_needed(engine.symbolic_for(*r.eps_r.shape), "c64", 8) for r in reqs)
    srv = SolveServer(slots=4, precision="c64", memory_budget=int(need * 1.5), cache_budget=0)
    s = srv.run(reqs, realtime=False)
    assert s["failed"] == 0 and srv.resident == 0
    big = _requests()[:1]
    small_budget = SolveServer(slots=2, precision="c64", memory_budget=1024, cache_budget=0)
    s = small_budget.run(big, realtime=False)
    assert s["failed"] == 1 and "memory" in big[0].error


def test_cached_factor_is_reused_for_new_sources():
    from fdfdpy_gb300.serving import SolveServer, Request
    base = _requests()[0]
    rng = np.random.default_rng(9)
    n = base.eps_r.size
    first = Request(eps_r=base.eps_r, rhs=base.rhs[:1], omega=base.omega, dl=base.dl, NPML=base.NPML,
                    pol=base.pol, arrival=0.0, rid=0)
    second = Request(eps_r=base.eps_r.copy(), rhs=rng.standard_normal((5, n)) + 1j * rng.standard_normal((5, n)),
                     omega=base.omega, dl=base.dl, NPML=base.NPML, pol=base.pol, arrival=0.5, rid=1)
    srv = SolveServer(slots=2, precision="c64", tol=1e-10)
    s = srv.run([first, second], realtime=True)
    assert s["failed"] == 0 and s["cache_hits"] == 1 and second.cache_hit
    assert second.x.shape == (5, n) and second.rel_residual <= 1e-10


def test_unconverged_request_is_solved_again_in_complex128():
    """A request whose complex64 refinement stops short of the tolerance
    (here: one refinement step against 1e-13) is solved again with a
    complex128 factor, flagged, and meets the tolerance."""
    from fdfdpy_gb300.serving import SolveServer
    reqs = _requests()[:3]
    srv = SolveServer(slots=2, precision="c64", tol=1e-13, max_iter=1)
    s = srv.run(reqs, realtime=False)
    assert s["failed"] == 0, [r.error for r in reqs if r.error]
    assert s["c128_fallbacks"] == len(reqs)
    for r in reqs:
        assert r.fallback and r.rel_residual <= 1e-13, (r.rid, r.rel_residual)


def test_tensor_core_requests_alone_equal_mix():
    """The served headline path (complex64 factor with the tensor-core Schur
    update, c64tc) on requests large enough to reach the tensor-core levels
    (fronts of 192 rows or more: 512^2 and 768^2 grids) mixed with small
    ones: every result meets the residual tolerance and equals the same
    request solved alone."""
    from fdfdpy_gb300.serving import SolveServer, make_stream
    from fdfdpy_gb300 import engine

    def reqs():
        rs = make_stream(n_requests=6, rate=1e6, sides=(128, 512, 768), reuse=0.2, seed=11, npml=(10, 10))
        for r in rs:
            r.arrival = 0.0
        return rs

    big = [r for r in reqs() if r.eps_r.shape[0] >= 512]
    assert big and max(engine.symbolic_for(*r.eps_r.shape).info.max_m for r in big) >= 192
    alone = {}
    for r in reqs():
        s = SolveServer(slots=1, precision="c64tc", tol=1e-10).run([r], realtime=False)
        assert s["failed"] == 0, r.error
        alone[r.rid] = r.x
    mix = reqs()
    s = SolveServer(slots=3, precision="c64tc", tol=1e-10, batch_max=1).run(mix, realtime=False)
    assert s["failed"] == 0, [r.error for r in mix if r.error]
    assert s["max_rel_residual"] <= 1e-10
    for r in mix:
        a = alone[r.rid]
        assert np.linalg.norm(r.x - a) <= 1e-12 * np.linalg.norm(a), r.rid


def test_batch_factor_matches_single_factors():
    """A forest factorization of several operators of one grid (every
    level's front updates of all of them in one launch) against the same
    operators factored one by one and against the oracle: residual <= 1e-10
    per (problem, right-hand side), fields within 1e-8; a problem with no
    right-hand sides stays zero; a cached batch entry serves a later hit."""
    import torch
    from oracle import fdfd_oracle as O
    from fdfdpy_gb300 import engine
    rng = np.random.default_rng(12)
    N, B = 96, 3
    om = 2 * np.pi * O.C_0 / 1.55e-6
    for pol, prec in (("Hz", "c64tc"), ("Ez", "c64"), ("Hz", "c128")):
        eps = [np.kron(rng.choice([1.0, 12.25], size=(N // 8, N // 8)), np.ones((8, 8))) for _ in range(B)]
        ops = [engine.DeviceOperator(om, e, N * 0.02, N * 0.02, [10, 10], pol, 1e-6) for e in eps]
        fac = engine.BatchFactor(engine.symbolic_for(N, N, batch=B), prec).numeric(ops)
        rhs = [rng.standard_normal((k, N * N)) + 1j * rng.standard_normal((k, N * N)) for k in (2, 5, 0)]
        xs, worst = fac.solve_batch(rhs, tol=1e-10, max_iter=40)
        assert max(worst) <= 1e-10 and worst[2] == 0.0 and xs[2].shape[0] == 0
        for p in range(2):
            single = engine.Factor(engine.symbolic_for(N, N), prec, max_nrhs=8).numeric(ops[p]).solve(
                engine.as_c128(rhs[p]), tol=1e-10, max_iter=40).cpu().numpy()
            got = xs[p].cpu().numpy()
            A = O.construct_A(om, N * 0.02, N * 0.02, eps[p], [10, 10], pol, 1e-6)
            for k in range(rhs[p].shape[0]):
                assert np.linalg.norm(A @ got[k] - rhs[p][k]) <= 1.01e-10 * np.linalg.norm(rhs[p][k])
                assert np.linalg.norm(got[k] - single[k]) <= 1e-8 * np.linalg.norm(single[k])


def test_autotuner_picks_a_measured_candidate(tmp_path):
    """The project's autotuner times every (batch size, whole-front limit)
    candidate on the device, keeps the fastest, writes its table, and the
    server uses it (results still meet the tolerance)."""
    from fdfdpy_gb300.autotune import Autotuner
    from fdfdpy_gb300.serving import SolveServer, make_stream
    path = tmp_path / "tune.json"
    tuner = Autotuner(batches=(1, 2, 4), fused_limits=(-1, 0), nrhs=2, path=str(path))
    cfg = tuner.config_for((96, 96), "c64")
    cands = cfg["candidates"]
    assert len(cands) == 6 and all(c["ms"] > 0 for c in cands)
    assert cfg["solves_per_s"] == max(c["solves_per_s"] for c in cands)
    assert Autotuner(path=str(path)).batch_for((96, 96), "c64") == cfg["batch"]
    reqs = make_stream(n_requests=8, rate=1e6, sides=(96,), reuse=0.0, seed=4, npml=(8, 8))
    s = SolveServer(slots=2, precision="c64", autotune=tuner, batch_max=8).run(reqs, realtime=False)
    assert s["failed"] == 0 and s["max_rel_residual"] <= 1e-10


def test_failed_factorization_fails_its_requests_and_the_slot_goes_on(monkeypatch):
    """A factorization that raises inside a slot (here a simulated device
    allocation failure, raised on the host for one grid) fails exactly the
    requests of that unit of work; the slot is freed, the memory it had
    reserved is returned, and the other requests are served."""
    from fdfdpy_gb300 import engine, _native as N
    from fdfdpy_gb300.serving import SolveServer
    reqs = _requests()[:6]
    bad_shape = reqs[0].eps_r.shape
    real_init = engine.Factor.__init__

    def flaky_init(self, sym, *a, **k):
        if (sym.Nx, sym.Ny) == bad_shape:
            raise N.FDFDError(N.FDFD_ERR_OOM, "factor_create: device allocation failed")
        real_init(self, sym, *a, **k)

    monkeypatch.setattr(engine.Factor, "__init__", flaky_init)
    srv = SolveServer(slots=2, precision="c64", tol=1e-10, batch_max=1, cache_budget=0)
    s = srv.run(reqs, realtime=False)
    bad = [r for r in reqs if r.eps_r.shape == bad_shape]
    good = [r for r in reqs if r.eps_r.shape != bad_shape]
    assert bad and good
    assert s["failed"] == len(bad)
    assert all(r.error and "allocation" in r.error and r.x is None for r in bad)
    assert all(r.error is None and r.rel_residual <= 1e-10 for r in good)
    assert srv.resident == 0
