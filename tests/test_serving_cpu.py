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
