"""Host logic of the serving loop (no GPU): request streams, batch formation, summaries."""

from collections import deque
from types import SimpleNamespace

import numpy as np

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


def test_batch_formation_respects_busy_topologies_and_limits():
    topos = [_topo(grid_118()), _topo(make_grid(300, seed=3))]
    S0, S1 = np.zeros(118, complex), np.zeros(300, complex)
    reqs = [Request(0, 0, "single", 0.0, S0), Request(1, 1, "chunk", 0.1, np.zeros((300, 50), complex)),
            Request(2, 0, "chunk", 0.2, np.zeros((118, 40), complex)), Request(3, 1, "single", 0.3, S1),
            Request(4, 0, "n1", 0.4, S0, np.arange(20))]
    s = _server(topos, max_cases=60, budget=1e12)
    pending = deque(reqs)
    take, tp, mem = s._form(pending, busy_topos={1}, budget_left=1e12)
    # topology 1 is busy: its requests wait; topology 0 fills up to 60 cases in arrival order
    assert [r.rid for r in take] == [0, 2] and tp == {0}
    assert [r.rid for r in pending] == [1, 3, 4]
    assert mem == (1 + 40) * 1000 * 118
    # the memory budget admits the oldest request even when it alone exceeds the budget
    pending = deque(reqs)
    take, _, _ = _server(topos, 10_000, 1.0)._form(pending, set(), 1.0)
    assert [r.rid for r in take] == [0]


def test_latency_summary():
    rs = [Response(i, np.zeros((2, 1)), np.array([3]), np.array([True]), arrival=0.01 * i, start=0.0,
                   done=0.01 * i + 0.001 * (i + 1), launch=0) for i in range(100)]
    s = latency_summary(rs)
    assert s["requests"] == 100 and s["cases"] == 100 and s["converged_fraction"] == 1.0
    assert abs(s["p50_ms"] - 50.5) < 1e-6 and abs(s["p99_ms"] - 99.01) < 1e-6 and abs(s["max_ms"] - 100.0) < 1e-6
