"""Host logic of the serving loop (no GPU): request streams, batch formation, summaries."""

from collections import deque
from types import SimpleNamespace

import numpy as np
import pytest

from p3s_gb300.serving import Request, Response, Server, latency_summary, poisson_stream
from p3s_gb300.synthetic import grid_118, make_grid


def _topo(g):
    return SimpleNamespace(grid=g, n=g.n, nv=len(g.pv) + len(g.pq), nblk=4 * g.n, f=g.f,
                           slot_bytes=lambda mixed, n=g.n: 1000 * n)


def test_poisson_stream_mix_and_shapes():
    topos = [_topo(grid_118()), _topo(make_grid(300, seed=3))]
    reqs = poisson_stream(topos, rate=2000.0, duration=1.0, seed=4, chunk=8, n1_outages=10)
    assert 1700 < len(reqs) < 2300
    arr = np.array([r.arrival for r in reqs])
    assert (np.diff(arr) > 0).all() and arr[-1] <= 1.0
    kinds = np.array([r.kind for r in reqs])
    frac = [(kinds == k).mean() for k in ("single", "chunk", "n1")]
    assert abs(frac[0] - 0.70) < 0.05 and abs(frac[1] - 0.25) < 0.05 and abs(frac[2] - 0.05) < 0.02
    for r in reqs:
        n = topos[r.topo].n
        if r.kind == "single":
            assert r.S.shape == (n,)
        elif r.kind == "chunk":
            assert r.S.shape == (n, 8)
        else:
            assert len(r.outages) == 10 and len(np.unique(r.outages)) == 10
    again = poisson_stream(topos, rate=2000.0, duration=1.0, seed=4, chunk=8, n1_outages=10)
    assert [r.arrival for r in again] == list(arr)


def _server(topos, max_cases, budget):
    s = object.__new__(Server)
    s.topos, s.mixed, s.max_cases, s.hbm_budget = topos, True, max_cases, budget
    return s


def test_batch_formation_respects_case_and_memory_limits():
    topos = [_topo(grid_118()), _topo(make_grid(300, seed=3))]
    S0, S1 = np.zeros(118, complex), np.zeros(300, complex)
    reqs = [Request(0, 0, "single", 0.0, S0), Request(1, 1, "chunk", 0.1, np.zeros((300, 50), complex)),
            Request(2, 0, "chunk", 0.2, np.zeros((118, 40), complex)), Request(3, 1, "single", 0.3, S1),
            Request(4, 0, "n1", 0.4, S0, np.arange(20))]
    s = _server(topos, max_cases=60, budget=1e12)
    pending = deque(reqs)
    take, mem = s._form(pending, budget_left=1e12)
    # up to 60 cases in arrival order; a request that does not fit waits, later ones may fit
    assert [r.rid for r in take] == [0, 1, 3]
    assert [r.rid for r in pending] == [2, 4]
    assert mem == 1 * 1000 * 118 + 51 * 1000 * 300
    # the memory budget admits the oldest request even when it alone exceeds the budget
    pending = deque(reqs)
    take, _ = _server(topos, 10_000, 1.0)._form(pending, 1.0)
    assert [r.rid for r in take] == [0]
    # a small-request context takes requests of at most small_work bus-cases only
    s.small_work = 40 * 118
    pending = deque(reqs)
    take, _ = s._form(pending, 1e12, small_only=True)
    assert [r.rid for r in take] == [0, 2, 3] and [r.rid for r in pending] == [1, 4]


def test_jobs_keep_large_requests_in_place():
    topos = [_topo(grid_118()), _topo(make_grid(300, seed=3))]
    for tp in topos:
        tp.solver, tp.V_warm = None, np.ones(tp.n, complex)
        tp.n1_job = lambda outages, S, tp=tp: SimpleNamespace(solver=None, S=S, outages=outages)
    rng = np.random.default_rng(1)
    a, b, c = (rng.standard_normal(118) + 0j for _ in range(3))
    chunk = np.ascontiguousarray(rng.standard_normal((300, 7)) + 0j)
    reqs = [Request(0, 0, "single", 0.0, a), Request(1, 1, "chunk", 0.1, chunk),
            Request(2, 0, "single", 0.2, b), Request(3, 0, "n1", 0.3, c, np.arange(5)),
            Request(4, 1, "single", 0.4, np.zeros(300, complex))]
    s = _server(topos, max_cases=10_000, budget=1e12)
    jobs, layout, served = s._jobs(reqs)
    spans = [[(r.rid, lo, hi) for r, lo, hi in lay] for lay in layout]
    # chunk and N-1 alone (their arrays in place), the single solves of a topology together
    assert spans == [[(1, 0, 7)], [(3, 0, 5)], [(0, 0, 1), (2, 1, 2)], [(4, 0, 1)]]
    assert jobs[0].S is chunk and jobs[1].S is c and served == {3: True}
    assert np.array_equal(jobs[2].S, np.stack([a, b], axis=1))


def test_latency_summary():
    rs = [Response(i, np.zeros((2, 1)), np.array([3]), np.array([True]), arrival=0.01 * i, start=0.0,
                   done=0.01 * i + 0.001 * (i + 1), launch=0) for i in range(100)]
    s = latency_summary(rs)
    assert s["requests"] == 100 and s["cases"] == 100 and s["converged_fraction"] == 1.0
    assert abs(s["p50_ms"] - 50.5) < 1e-6 and abs(s["p99_ms"] - 99.01) < 1e-6 and abs(s["max_ms"] - 100.0) < 1e-6


class _FakeGroup:
    """Stands in for a launch context: results are the job's S columns (n1: the base S per
    outage), one iteration each."""

    def __init__(self):
        self.calls = []

    def solve(self, jobs, params, pinned_out=False):
        self.calls.append(len(jobs))
        out = []
        for j in jobs:
            T = j.n_cases or (j.S.shape[1] if j.S.ndim == 2 else 1)
            V = np.repeat(j.S[:, None], T, axis=1) if j.S.ndim == 1 else j.S.copy()
            r = {"V": V, "iterations": np.ones(T, np.int32), "converged": np.ones(T, bool)}
            if j.outages is not None:
                r["served"] = np.ones(V.shape, bool)
            out.append(r)
        return out


@pytest.mark.parametrize("keep", [True, False])
def test_serving_loop_delivers_every_request(keep):
    import threading

    topos = [_topo(grid_118()), _topo(make_grid(300, seed=3))]
    for tp in topos:
        tp.solver, tp.V_warm = SimpleNamespace(n=tp.n), np.ones(tp.n, complex)
        tp.n1_job = lambda outages, S, tp=tp: SimpleNamespace(solver=tp.solver, S=S, n_cases=len(outages),
                                                              outages=(None, outages))
    reqs = poisson_stream(topos, rate=4000.0, duration=0.05, seed=2, chunk=5, n1_outages=4)
    s = _server(topos, max_cases=64, budget=1e12)
    s.groups = [_FakeGroup(), _FakeGroup()]
    s.small, s.small_work, s.params, s.pinned_results = {1}, 10_000, None, False
    s._cv = threading.Condition()
    resp = s.run(reqs, realtime=False, keep_results=keep)
    assert [r.rid for r in resp] == [q.rid for q in reqs]
    for q, r in zip(reqs, resp):
        T = len(q.outages) if q.kind == "n1" else (1 if q.S.ndim == 1 else q.S.shape[1])
        assert len(r.iterations) == T and r.converged.all() and r.done >= r.start >= 0.0
        if keep:
            want = np.repeat(q.S[:, None], T, axis=1) if q.kind != "chunk" else q.S
            assert np.array_equal(r.V, want) and (r.served is not None) == (q.kind == "n1")
        else:
            assert r.V is None and r.served is None
    assert sum(sum(g.calls) for g in s.groups) >= len({r.launch for r in resp})


class _FakeStream:
    """Stand-in for a stream launch: a job's results (V = its request's S, iterations 3) are
    ready `delay` polls after its submit; at most `capacity` jobs per launch."""

    def __init__(self, capacity, delay=2, die_after=None):
        self.capacity, self.delay, self.die_after = capacity, delay, die_after
        self.starts, self.stops, self.polls = 0, 0, 0

    def start(self, solvers, params, idle_seconds):
        self.starts += 1
        self.jobs, self.flag = [], np.zeros(self.capacity, np.int32)
        self.running = True
        self.launch_polls = 0

    def submit(self, solver, S, V0, outages=None, reslack=True, precision=None):
        assert self.running
        self.precisions = getattr(self, "precisions", []) + [precision]
        if len(self.jobs) == self.capacity:
            return None
        T = S.shape[1] if S.ndim == 2 else 1
        outs = (np.array(S).reshape(-1, T).copy(), np.full(T, 3, np.int32), np.ones(T, np.uint8),
                np.ones((len(V0), T), np.uint8) if outages is not None else None)
        self.jobs.append(self.polls)
        return len(self.jobs) - 1, outs

    def _dead(self):  # only the first launch reaches its idle limit, after die_after polls
        return self.die_after is not None and self.starts == 1 and self.launch_polls >= self.die_after

    def flags(self):
        if self.running and not self._dead():
            self.polls += 1
            self.launch_polls += 1
            for q, t in enumerate(self.jobs):
                if self.polls - t >= self.delay:
                    self.flag[q] = 1
        return self.flag

    def done(self, q):
        return bool(self.flag[q])

    def full(self):
        return len(self.jobs) == self.capacity

    def release(self, q):
        self.released = getattr(self, "released", 0) + 1

    def alive(self):
        return not self._dead()

    def stop(self):
        self.stops += 1
        self.running = False
        if self._dead():  # returned at its idle limit: unstarted jobs keep flag 0
            return 1
        self.flag[:len(self.jobs)] = 1
        return 0


def _stream_server(topos, backend):
    from p3s_gb300.serving import StreamServer

    s = object.__new__(StreamServer)
    s.topos, s.params, s.idle_seconds, s.backend, s.launches = topos, None, 1.0, backend, 0
    s.precision_of = {}
    return s


def test_stream_server_admits_as_requests_arrive_and_restarts_a_full_launch():
    topos = [SimpleNamespace(solver=None, V_warm=np.ones(118, complex), grid=grid_118(), n=118)]
    reqs = [Request(i, 0, "single" if i % 3 else "chunk", 0.0,
                    np.full((118,) if i % 3 else (118, 4), i + 1.0, complex)) for i in range(10)]
    reqs.append(Request(10, 0, "n1", 0.0, np.zeros(118, complex), np.arange(5)))
    fake = _FakeStream(capacity=3)
    srv = _stream_server(topos, fake)
    out = srv.run(reqs, realtime=False)
    assert [r.rid for r in out] == list(range(11))
    assert fake.starts == 4 and fake.stops == 4  # 11 jobs, 3 per launch
    for r, resp in zip(reqs, out):
        assert np.array_equal(resp.V.reshape(r.S.shape) if r.kind != "n1" else resp.V[:, 0], r.S if r.kind != "n1"
                              else np.zeros(118))
        assert (resp.iterations == 3).all() and resp.converged.all() and resp.done >= resp.start
    assert out[10].served is not None and out[10].served.all()
    assert {r.launch for r in out} == {0, 1, 2, 3}


def test_stream_server_resubmits_the_jobs_a_launch_left_at_its_idle_limit():
    """A launch whose CTAs left at their idle limit before some jobs were published: the
    server stops it (status 1), keeps the finished jobs' results and submits the unstarted
    ones again, in order, to a new launch."""
    topos = [SimpleNamespace(solver=None, V_warm=np.ones(118, complex), grid=grid_118(), n=118)]
    reqs = [Request(i, 0, "single", 0.0, np.full(118, i + 1.0, complex)) for i in range(3)]
    fake = _FakeStream(capacity=8, delay=4, die_after=3)
    srv = _stream_server(topos, fake)
    out = srv.run(reqs, realtime=False)
    assert fake.starts == 2 and fake.stops == 2
    assert [r.launch for r in out] == [1, 1, 1]  # none finished in the first launch
    for r, resp in zip(reqs, out):
        assert np.array_equal(resp.V[:, 0], r.S) and resp.converged.all()


def test_stream_server_tunes_the_precision_per_topology_and_kind():
    """``tune`` times each request kind of each topology (a few copies together) in the running
    launch in both precisions and keeps the faster; later requests are submitted with that
    precision."""

    class Timed(_FakeStream):
        def submit(self, solver, S, V0, outages=None, reslack=True, precision=None):
            sub = super().submit(solver, S, V0, outages, reslack, precision)
            kind = "n1" if outages is not None else ("chunk" if S.ndim == 2 else "single")
            slow = "mixed" if kind == "n1" else "double"  # this stand-in's slower precision per kind
            if sub is not None and precision == slow:
                self.jobs[-1] += 300  # its flag comes 300 polls later
            return sub

    topos = [SimpleNamespace(solver=None, V_warm=np.ones(118, complex), grid=grid_118(), n=118)]
    fake = Timed(capacity=64)
    srv = _stream_server(topos, fake)
    srv.params = SimpleNamespace(precision=1)  # a mixed-precision launch
    got = srv.tune(chunk=4, n1_outages=3, repeats=2)
    assert got == {(0, "single"): "mixed", (0, "chunk"): "mixed", (0, "n1"): "double"}
    fake.precisions = []
    reqs = [Request(0, 0, "single", 0.0, np.ones(118, complex)),
            Request(1, 0, "n1", 0.0, np.ones(118, complex), np.array([1, 2], np.int32))]
    srv.run(reqs, realtime=False)
    assert fake.precisions == ["mixed", "double"]
    srv.params = SimpleNamespace(precision=0)  # a double launch: nothing to choose
    assert srv.tune() == {}


def test_stream_server_reports_a_stopped_launch_with_jobs_unfinished():
    class Broken(_FakeStream):
        def stop(self):
            self.stops += 1
            self.running = False
            return 0  # a clean stop must leave no job unfinished

    topos = [SimpleNamespace(solver=None, V_warm=np.ones(118, complex), grid=grid_118(), n=118)]
    reqs = [Request(0, 0, "single", 0.0, np.ones(118, complex))]
    srv = _stream_server(topos, Broken(capacity=4, delay=10 ** 9, die_after=3))
    with pytest.raises(RuntimeError, match="unfinished"):
        srv.run(reqs, realtime=False)


def test_stream_result_memory_is_reused_in_job_order_and_refuses_when_full():
    """The stream launch's circular result memory: blocks in job order, refused while every
    byte is held by unconsumed jobs, given back in job order (a later job's release waits for
    the older ones), reused across the wrap; a block taken for a job that was then not
    submitted is given back at once."""
    from p3s_gb300 import stream

    class Slab(stream._Slab):
        def __init__(self, n):
            self.nbytes, self.buf = n, bytearray(n)
            self.reset()

        def __del__(self):
            pass

    f8 = np.float64
    s = Slab(4096)
    assert s.take(0, [((100,), f8)]) is not None and s.take(1, [((200,), f8)]) is not None
    assert s.take(2, [((150,), f8)]) is not None and s.head == 4096
    assert s.take(3, [((10,), f8)]) is None  # full
    s.release(1)
    assert s.tail == 0  # job 0 still holds the front
    s.release(0)
    assert s.tail == 2816
    v = s.take(3, [((100,), f8), ((4,), np.int32)])
    assert v is not None and s.wrapped and s.head == 1024 + 256 and v[0].shape == (100,) and v[1].dtype == np.int32
    s.undo(3)
    assert s.head == 4096 and not s.wrapped
    assert s.take(3, [((100,), f8)]) is not None and s.wrapped
    s.release(2)
    s.release(3)
    assert s.order == [] and s.head == s.tail
    with pytest.raises(ValueError, match="exceed the result memory"):
        s.take(4, [((1000,), f8)])
