"""The serving loop's host logic on a CPU: arrivals, FIFO admission by slots
and byte budget, continuous stepping, retirement and latency accounting,
against a fake session with a fake clock (no GPU)."""
import numpy as np
import pytest

from qsm_gb300 import serve
from qsm_gb300._lib import QsmError


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


class FakeSession:
    """Primal-dual jobs finish after `maxiter` stepped iterations (each step
    costs `step_cost` seconds per running job); Poisson jobs after
    `poisson_time` seconds.  Footprint = voxels * bytes per kind."""

    BPV = {"poisson": 40, "tv": 63, "tgv": 147}

    def __init__(self, clock, budget, step_cost=1e-4, poisson_time=0.02, fail_kind=None):
        self.clock, self.budget = clock, budget
        self.step_cost, self.poisson_time = step_cost, poisson_time
        self.jobs, self.next_id, self.used, self.max_used = {}, 1, 0, 0
        self.admit_order = []
        self.fail_kind = fail_kind

    def _admit(self, kind, shape, maxiter, payload):
        if kind == self.fail_kind:
            raise QsmError(5, "fake CUDA failure")
        b = int(np.prod(shape)) * self.BPV[kind]
        if self.budget and self.used + b > self.budget:
            raise QsmError(8, "session byte budget exceeded")
        jid = self.next_id
        self.next_id += 1
        self.used += b
        self.max_used = max(self.max_used, self.used)
        self.jobs[jid] = dict(kind=kind, bytes=b, left=maxiter, t0=self.clock(), payload=payload, iters=0)
        self.admit_order.append(jid)
        return jid

    def submit_pd(self, d2f, mask, vsz, lam, alpha, tol, maxiter, *, tgv=True):
        return self._admit("tgv" if tgv else "tv", d2f.shape, maxiter, d2f)

    def submit_mgpcg(self, v, f, mask, vsz, *args, mixed=True):
        return self._admit("poisson", f.shape, 0, f)

    def step(self, iters):
        run = [j for j in self.jobs.values() if j["kind"] != "poisson" and j["left"] > 0]
        self.clock.t += self.step_cost * len(run) * iters / 30
        for j in run:
            n = min(iters, j["left"])
            j["left"] -= n
            j["iters"] += n

    def poll(self, jid):
        j = self.jobs[jid]
        if j["kind"] == "poisson":
            return self.clock() - j["t0"] >= self.poisson_time, dict(iters=3)
        return j["left"] <= 0, dict(iters=j["iters"])

    def fetch(self, jid):
        j = self.jobs.pop(jid)
        self.used -= j["bytes"]
        return j["payload"] * 2.0

    def running(self):
        return len(self.jobs)


class PackedFakeSession(FakeSession):
    """A session without Poisson workers: Poisson jobs advance only in
    step(), one PCG iteration per step, `poisson_iters` in all."""

    poisson_workers = 0

    def __init__(self, clock, budget, poisson_iters=5, **kw):
        super().__init__(clock, budget, **kw)
        self.poisson_iters = poisson_iters

    def submit_mgpcg(self, v, f, mask, vsz, *args, mixed=True):
        return self._admit("poisson", f.shape, self.poisson_iters, f)

    def step(self, iters):
        super().step(iters)
        for j in self.jobs.values():
            if j["kind"] == "poisson" and j["left"] > 0:
                j["left"] -= 1
                j["iters"] += 1
        self.clock.t += self.step_cost

    def poll(self, jid):
        j = self.jobs[jid]
        if j["kind"] == "poisson":
            return j["left"] <= 0, dict(iters=j["iters"])
        return super().poll(jid)


def _pool():
    rng = np.random.default_rng(0)
    pool = {}
    for kind, shapes in (("poisson", [(20, 20, 20), (30, 24, 20)]), ("tv", [(24, 24, 16), (32, 24, 24)]),
                         ("tgv", [(24, 20, 16), (40, 32, 24)])):
        pool[kind] = []
        for s in shapes:
            a = np.asfortranarray(rng.standard_normal(s).astype(np.float32))
            m = np.ones(s, np.uint8, order="F")
            pool[kind].append(dict(shape=s, d2f=a, f=a.astype(np.float64), mask=m))
    return pool


def test_arrivals_poisson_process():
    a = serve.arrivals(4.0, 600.0, seed=4, pool_size=8)
    assert a == serve.arrivals(4.0, 600.0, seed=4, pool_size=8)  # seeded
    assert 2200 < len(a) < 2600  # 2400 +- 4 sigma
    t = np.array([r.t_arrive for r in a])
    assert np.all(np.diff(t) > 0) and t[-1] < 600.0
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 0.25) < 0.02
    frac = {k: sum(r.kind == k for r in a) / len(a) for k in serve.KINDS}
    assert abs(frac["poisson"] - 0.4) < 0.04 and abs(frac["tv"] - 0.3) < 0.04 and abs(frac["tgv"] - 0.3) < 0.04
    assert {r.case for r in a} == set(range(8))


def test_lbv_args():
    a = serve.lbv_args((176, 160, 112))
    assert a["maxitcg"] == int(np.ceil(np.sqrt(176 * 160 * 112)))
    assert (a["tolcg"], a["maxitmg"], a["npre"], a["npost"], a["nboundary"], a["mu"], a["nlevels"]) == \
        (1e-8, 2, 2, 2, 2, 1, 5)


def _run(budget, max_active=64, rate=40.0, duration=2.0, **kw):
    clock = FakeClock()
    pool = _pool()
    s = FakeSession(clock, budget, **kw)
    loop = serve.ServeLoop(s, {k: [dict(c) for c in v] for k, v in pool.items()}, max_active=max_active,
                           clock=clock, sleep=clock.sleep, keep_results=True)
    reqs = serve.arrivals(rate, duration, seed=1, pool_size=2)
    # the loop reads maxiter from the solver arguments: make them small
    serve_tv, serve_tgv = dict(serve.TV_ARGS), dict(serve.TGV_ARGS)
    try:
        serve.TV_ARGS["maxiter"], serve.TGV_ARGS["maxiter"] = 90, 150
        recs = loop.run(reqs)
    finally:
        serve.TV_ARGS.update(serve_tv)
        serve.TGV_ARGS.update(serve_tgv)
    return loop, s, reqs, recs


def test_loop_retires_every_request_in_fifo_order():
    loop, s, reqs, recs = _run(budget=0)
    assert len(recs) == len(reqs) and s.used == 0 and not s.jobs
    by_rid = {r.rid: r for r in recs}
    admits = [by_rid[q.rid].t_admit for q in sorted(reqs, key=lambda q: q.t_arrive)]
    assert np.all(np.diff(admits) >= 0)  # FIFO admission
    for r in recs:
        assert r.t_arrive <= r.t_admit <= r.t_done
        if r.kind == "tv":
            assert r.iters == 90
        if r.kind == "tgv":
            assert r.iters == 150
    assert loop.steps > 0 and loop.max_resident > 1  # requests overlapped (continuous batching)
    # the same (kind, case) always returns the same result
    for r in recs:
        assert r.digest == serve.digest(loop.results[(r.kind, r.case)])


def test_budget_limits_resident_bytes_and_requests_wait():
    big = 40 * 32 * 24 * 147
    loop, s, reqs, recs = _run(budget=big + 20 * 20 * 20 * 40, rate=200.0, duration=0.5)
    assert len(recs) == len(reqs)
    assert s.max_used <= big + 20 * 20 * 20 * 40
    assert loop.refusals > 0 and loop.max_queue > 1


def test_request_larger_than_budget_is_rejected_not_waited_on():
    loop, s, reqs, recs = _run(budget=30 * 24 * 20 * 40, rate=20.0, duration=1.0)
    big = [q for q in reqs if q.kind in ("tv", "tgv") and q.case == 1]
    assert big and {q.rid for q in loop.rejected} >= {q.rid for q in big}
    assert len(recs) + len(loop.rejected) == len(reqs)


def test_slot_limit():
    loop, s, reqs, recs = _run(budget=0, max_active=2, rate=200.0, duration=0.5)
    assert len(recs) == len(reqs)
    assert loop.max_resident <= 2


def test_non_budget_errors_propagate():
    with pytest.raises(QsmError, match="CUDA"):
        _run(budget=0, fail_kind="tgv")


def test_summarize():
    recs = [serve.Record(i, "tv", 0, (8, 8, 8), 0.0, 0.0, (i + 1) * 0.01, "", 10) for i in range(100)]
    out = serve.summarize(recs, duration=1.0)
    assert out["requests"] == 100
    assert abs(out["p50_ms"] - 505.0) < 1e-6 and abs(out["p99_ms"] - 990.1) < 1e-6
    assert out["tv"]["n"] == 100 and "tgv" not in out
    assert abs(out["throughput_rps"] - 100.0) < 1e-9


def test_loop_steps_packed_poisson_without_pd_jobs():
    """A session without Poisson workers advances its Poisson solves only in
    its steps: the loop steps whenever anything is resident, so a stream of
    Poisson requests alone is served (and mixed with primal-dual ones)."""
    clock = FakeClock()
    pool = _pool()
    s = PackedFakeSession(clock, 0, poisson_iters=7)
    loop = serve.ServeLoop(s, pool, clock=clock, sleep=clock.sleep)
    reqs = [serve.Request(i, 0.01 * i, "poisson", i % 2) for i in range(10)]
    recs = loop.run(reqs)
    assert len(recs) == 10 and all(r.iters == 7 for r in recs)
    assert loop.steps >= 7 and not s.jobs
    # mixed with primal-dual requests, every request still retires
    clock = FakeClock()
    s = PackedFakeSession(clock, 0, poisson_iters=4)
    loop = serve.ServeLoop(s, {k: [dict(c) for c in v] for k, v in pool.items()}, clock=clock, sleep=clock.sleep)
    reqs = serve.arrivals(40.0, 1.0, seed=2, pool_size=2)
    saved = dict(serve.TV_ARGS), dict(serve.TGV_ARGS)
    try:
        serve.TV_ARGS["maxiter"], serve.TGV_ARGS["maxiter"] = 60, 90
        recs = loop.run(reqs)
    finally:
        serve.TV_ARGS.update(saved[0])
        serve.TGV_ARGS.update(saved[1])
    assert len(recs) == len(reqs) and not s.jobs
    assert all(r.iters == 4 for r in recs if r.kind == "poisson")
