"""Serving loop on the GPU: continuous batching over resident topologies. Each request's
result is the same alone and in the mix (bar: bit for bit -- every case runs the same
arithmetic whatever it is batched with), N-1 requests keep the islanding semantics, and
the mixed path stays within 1e-9 of the converged double solution."""

import numpy as np
import pytest

from p3s_gb300.serving import Server, Topology, latency_summary, poisson_stream
from p3s_gb300.synthetic import grid_118, make_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def topos():
    grids = [grid_118(), make_grid(400, seed=21), make_grid(1500, seed=22), make_grid(5000, seed=23)]
    return [Topology(g) for g in grids]


def test_results_are_the_same_alone_and_in_the_mix(topos):
    reqs = poisson_stream(topos, rate=400.0, duration=0.25, seed=5, chunk=12, n1_outages=24,
                          mix=(0.6, 0.3, 0.1))
    kinds = {r.kind for r in reqs}
    assert kinds == {"single", "chunk", "n1"}
    server = Server(topos, precision="mixed", contexts=2)
    server.warmup(cases=8)
    mixed_run = server.run(reqs, realtime=True)
    summary = latency_summary(mixed_run)
    assert summary["converged_fraction"] == 1.0 and summary["requests"] == len(reqs)
    launches = {r.launch for r in mixed_run}
    assert len(launches) < len(reqs)  # requests were batched together
    alone = Server(topos, precision="mixed", contexts=1)
    for r, got in zip(reqs, mixed_run):
        ref = alone.run([r], realtime=False)[0]
        assert np.array_equal(got.iterations, ref.iterations) and np.array_equal(got.converged, ref.converged)
        assert np.array_equal(np.isnan(got.V), np.isnan(ref.V))
        assert np.array_equal(np.nan_to_num(got.V), np.nan_to_num(ref.V))
        if r.kind == "n1":
            assert np.array_equal(got.served, ref.served) and (~got.served).sum() >= 0


def test_served_mixed_results_match_the_converged_double_solution(topos):
    reqs = poisson_stream(topos, rate=200.0, duration=0.2, seed=9, chunk=8, n1_outages=16, mix=(0.5, 0.4, 0.1))
    mixed = Server(topos, precision="mixed").run(reqs, realtime=False)
    tight = Server(topos, precision="double", tol=1e-12).run(reqs, realtime=False)
    for a, b in zip(mixed, tight):
        assert np.array_equal(a.converged, b.converged)
        ok = a.converged
        if ok.any():
            assert np.nanmax(np.abs(a.V[:, ok] - b.V[:, ok])) < 1e-9


def test_stream_launch_results_are_the_same_alone_and_in_the_mix(topos):
    """Slot-level admission: one running launch takes every request as it arrives; each result
    equals the request's own launch bit for bit (also N-1 islanding)."""
    from p3s_gb300.serving import StreamServer

    reqs = poisson_stream(topos, rate=400.0, duration=0.3, seed=7, chunk=12, n1_outages=24, mix=(0.6, 0.3, 0.1))
    assert {r.kind for r in reqs} == {"single", "chunk", "n1"}
    srv = StreamServer(topos, precision="mixed", capacity=64, arena_bytes=1 << 30, result_bytes=256 << 20)
    got = srv.run(reqs, realtime=True)
    assert srv.launches >= 2  # the 64-job ring was refilled by a new launch
    alone = Server(topos, precision="mixed", contexts=1)
    for r, g in zip(reqs, got):
        ref = alone.run([r], realtime=False)[0]
        assert np.array_equal(g.iterations, ref.iterations) and np.array_equal(g.converged, ref.converged)
        assert np.array_equal(np.isnan(g.V), np.isnan(ref.V)) and np.array_equal(np.nan_to_num(g.V),
                                                                                   np.nan_to_num(ref.V))
        if r.kind == "n1":
            assert np.array_equal(g.served, ref.served)
    assert latency_summary(got)["converged_fraction"] == 1.0


def test_stream_jobs_take_their_own_precision(topos):
    """In a mixed-precision stream launch a job may ask for double factors (and one for mixed,
    or the launch's): each result equals, bit for bit, that precision's own launch; a launch
    started in double refuses a mixed job."""
    import time

    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.stream import GpuStream

    tp = topos[2]
    pm = GpuSolver.params(precision="mixed", shared_start=False)
    pd = GpuSolver.params(precision="double", shared_start=False)
    S = tp.grid.Sbus
    # (before the launch: while a stream launch runs it holds the SMs, and another launch waits)
    ref = {"mixed": tp.solver.solve_batch(S[:, None], tp.V_warm, pm),
           "double": tp.solver.solve_batch(S[:, None], tp.V_warm, pd)}
    st = GpuStream(capacity=8, arena_bytes=256 << 20, result_bytes=64 << 20)
    st.start([tp.solver], pm, idle_seconds=10.0)
    jobs = [(st.submit(tp.solver, S, tp.V_warm, precision=pr), want)
            for pr, want in ((None, "mixed"), ("double", "double"), ("mixed", "mixed"))]
    t = time.perf_counter()
    while not all(st.flags()[j[0]] for j, _ in jobs) and time.perf_counter() - t < 20.0:
        time.sleep(0.001)
    assert all(st.done(j[0]) for j, _ in jobs)
    for (_, (V, it, cv, _)), want in jobs:
        assert np.array_equal(V, ref[want]["V"]) and np.array_equal(it, ref[want]["iterations"]) and cv.all()
    assert st.stop() == 0
    st.start([tp.solver], pd, idle_seconds=10.0)
    with pytest.raises(RuntimeError, match="precision"):
        st.submit(tp.solver, S, tp.V_warm, precision="mixed")
    assert st.stop() == 0


def test_stream_launch_returns_at_its_idle_limit_and_starts_again(topos):
    """A launch that gets no job for its idle window returns by itself (status 1 at stop) --
    its polling is bounded; a full ring refuses the next job until the launch is restarted."""
    import time

    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.stream import GpuStream

    tp = topos[1]
    p = GpuSolver.params(precision="double", shared_start=False)
    st = GpuStream(capacity=2, arena_bytes=64 << 20, result_bytes=16 << 20)
    st.start([tp.solver], p, idle_seconds=0.05)
    t = time.perf_counter()
    while st.alive() and time.perf_counter() - t < 20.0:
        time.sleep(0.01)
    assert not st.alive()
    assert st.stop() == 1
    S = tp.grid.Sbus
    # (before the launch: while a stream launch runs it holds the SMs, and another launch waits)
    ref = tp.solver.solve_batch(S[:, None], tp.V_warm, p)
    st.start([tp.solver], p, idle_seconds=10.0)
    jobs = [st.submit(tp.solver, S, tp.V_warm) for _ in range(2)]
    assert all(j is not None for j in jobs)
    assert st.submit(tp.solver, S, tp.V_warm) is None  # ring full
    t = time.perf_counter()
    while not all(st.flags()[q] for q, _ in jobs) and time.perf_counter() - t < 20.0:
        time.sleep(0.001)
    assert all(st.done(q) for q, _ in jobs)
    for _, (V, it, cv, _) in jobs:
        assert np.array_equal(V, ref["V"]) and np.array_equal(it, ref["iterations"]) and cv.all()
    assert st.stop() == 0
