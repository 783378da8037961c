"""GPU parity at the full sizes of the benchmarked workloads, every case compared.

* the 2,000-bus grid's 8,760-hour series, as the benchmark solves it (every hour from the
  converged base case), and in 12-hour warm-start lanes (K = 730);
* the full N-1 sweep of that grid (3,001 cases, islands re-slacked), both precisions;
* the uneven multi-grid batch's grids of 15,000 buses and more (16 scenarios each, one launch);
* the serving pool's three largest topologies (26,473 / 42,589 / 49,744 buses): a single solve,
  a 96-step chunk and a 200-outage sweep each, through the serving loop.

Bars, as in the reference's own full-case GPU test (tests/cuda/test_lean_lu.py:128-326): the
plain double path reproduces the oracle's iteration counts and convergence flags exactly and
its voltages to 1e-11 p.u. (N-1: 1e-10, the oracle rebuilds each case's Ybus from |Y| and
angle; grids of 15,000 buses and more: twice the distance between the reference's own release
and strict-IEEE builds on that grid, golden_floor.json, 1.6e-11 .. 6.1e-11); the mixed path converges on the same cases, every result's mismatch is at most 1e-8
p.u. and its voltages are within 1e-9 of the oracle solved to convergence (tol 1e-12); island
labels, served masks and reference buses are bit-exact.
"""

import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import cpu
from oracle import islands as oisl
from oracle.build import build_oracle

pytestmark = pytest.mark.gpu
TOL_V = 1e-11        # double path vs the oracle (p.u.)
TOL_V_N1 = 1e-10     # double path vs the oracle on outage cases (per-case Ybus from |Y|, angle)
TOL_V_MIXED = 1e-9   # mixed path vs the oracle solved to convergence
TOL_MISMATCH = 1e-8  # mismatch of every mixed result (p.u.)


def setup_module(_):
    build_oracle()


def double_tol(n, base=TOL_V):
    """The double path's bar on an n-bus grid (or a named stressed case): `base`, or on the
    large grids and near the loading limit twice the spread of the reference's own two builds
    there (golden_floor.json, made by make_golden_floor.py)."""
    with open(os.path.join(os.path.dirname(__file__), "golden", "golden_floor.json")) as fh:
        floor = json.load(fh)
    return max(base, 2.0 * floor.get(str(n), 0.0))


def _serving_sizes():
    """Bus counts of the serving pool's 32 topologies (sorted; topology i has seed 500 + i)."""
    rng = np.random.default_rng(5)
    return np.sort(np.exp(rng.uniform(np.log(100), np.log(50000), 32)).astype(int))


def mismatch(g, V, S, Yx=None, pin=None):
    """Infinity norm per column of the reference's F(V) = [P - Psp (pv, pq); Q - Qsp (pq)]
    (nr_klu.cpp:311-424), for all columns at once; Yx (nnz, L) per-case values if given.
    Pinned buses (re-slack references, unserved buses: identity rows, F = 0, nr_klu.cpp:398-423)
    are left out."""
    n = g.n
    V = np.where(np.isnan(V), 0.0, V)
    if Yx is None:
        Y = sp.csr_matrix((g.Yx, g.Yj, g.Yp), shape=(n, n))
        I = Y @ V
    else:
        rows = np.repeat(np.arange(n), np.diff(g.Yp))
        I = np.zeros_like(V)
        for c in range(V.shape[1]):
            I[:, c] = np.bincount(rows, weights=(Yx[:, c] * V[g.Yj, c]).real, minlength=n) + 1j * np.bincount(
                rows, weights=(Yx[:, c] * V[g.Yj, c]).imag, minlength=n)
    F = V * np.conj(I) - S
    if pin is not None:
        F = np.where(pin != 0, 0.0, F)
    pvpq = np.concatenate([g.pv, g.pq])
    return np.maximum(np.abs(F[pvpq].real).max(axis=0), np.abs(F[g.pq].imag).max(axis=0))


def converged_base(g, osv):
    r = osv.solve_batch(g.Sbus[:, None], g.V0)
    assert r["converged"][0]
    return np.ascontiguousarray(r["V"][:, 0])


def check_double(got, ref, tol=TOL_V):
    assert np.array_equal(got["converged"], ref["converged"])
    assert np.array_equal(got["iterations"], ref["iterations"])
    ok = ref["converged"]
    assert np.nanmax(np.abs(got["V"][:, ok] - ref["V"][:, ok])) < tol


def check_converged(got, ref, tol=TOL_V):
    """Flags equal on every case; iterations and voltages on the converged ones."""
    assert np.array_equal(got["converged"], ref["converged"])
    ok = ref["converged"]
    assert np.array_equal(got["iterations"][ok], ref["iterations"][ok])
    assert np.nanmax(np.abs(got["V"][:, ok] - ref["V"][:, ok])) < tol


def check_mixed(got, ref, tight, mis):
    assert np.array_equal(got["converged"], ref["converged"])
    assert (tight["converged"] | ~ref["converged"]).all()  # the oracle converges tight where it converges
    ok = ref["converged"] & tight["converged"]
    assert np.nanmax(np.abs(got["V"][:, ok] - tight["V"][:, ok])) < TOL_V_MIXED
    assert (mis[got["converged"]] <= TOL_MISMATCH).all()


def test_headline_series_every_hour(grid2000):
    """All 8,760 hours of the benchmarked series, each starting from the converged base case
    (one launch, K = T), then in 12-hour warm-start lanes (K = 730) against the oracle's
    replay of the same lanes."""
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.synthetic import lanes, timeseries_injections

    g = grid2000
    S = timeseries_injections(g, 8760, seed=1)
    osv = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    V0 = converged_base(g, osv)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    for K in (8760, 730):
        off = lanes(8760, K)
        ref = cpu.solve_lanes(osv, S, V0, off)
        tight = cpu.solve_lanes(osv, S, V0, off, tol=1e-12)
        assert ref["converged"].all() and tight["converged"].all()
        dbl = s.solve_lanes(S, V0, off, GpuSolver.params(precision="double"))
        check_double(dbl, ref)
        mixed = s.solve_lanes(S, V0, off, GpuSolver.params(precision="mixed"))
        check_mixed(mixed, ref, tight, mismatch(g, mixed["V"], S))
        if K < 8760:
            assert mixed["iterations"].mean() < ref["iterations"].mean() + 1.5  # warm starts pay off


def test_full_n1_sweep_every_case(grid2000):
    """The base case and all 3,000 single-branch outages: islands bit-exact, then every solve
    of both precisions against the oracle on per-case Ybus values and the same starts / pins."""
    from p3s_gb300 import contingency
    from p3s_gb300.cuda.nr_polar_solver import PolarNewtonSolverCUDA

    g = grid2000
    batch = contingency.build_batch(g)
    prio = np.zeros(g.n)
    prio[g.pv] = np.maximum(g.p_gen[g.pv], np.finfo(float).tiny)
    olab, osv_, orb, oni = oisl.islands(g.n, g.f, g.t, batch.live, batch.groups, g.ref, True, prio)
    V0, pin = oisl.start_and_pins(g.V0, osv_, orb, g.ref)
    Yx = batch.Yx_matrix
    osolver = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    mag, ang = np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx))
    ref = osolver.solve_batch_contingency(mag, ang, g.Sbus, V0, pin)
    tight = osolver.solve_batch_contingency(mag, ang, g.Sbus, V0, pin, tol=1e-12)
    ref["V"] = np.where(osv_, ref["V"], np.nan)
    tight["V"] = np.where(osv_, tight["V"], np.nan)
    assert ref["converged"].all()
    solver = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    res = contingency.solve_contingencies(g, reslack_islands=True, precision="double", solver=solver)
    assert np.array_equal(res.labels, olab) and np.array_equal(res.served, osv_)
    assert np.array_equal(res.ref_bus, orb)
    assert np.array_equal(np.isnan(res.V), ~osv_)
    check_double({"V": res.V, "iterations": res.iterations, "converged": res.converged}, ref, TOL_V_N1)
    mixed = contingency.solve_contingencies(g, reslack_islands=True, precision="mixed", solver=solver,
                                            return_islands=False)
    assert np.array_equal(mixed.served, osv_)
    got = {"V": mixed.V, "iterations": mixed.iterations, "converged": mixed.converged}
    check_mixed(got, ref, tight,
                mismatch(g, mixed.V, np.repeat(g.Sbus[:, None], len(batch.groups), axis=1), Yx, pin))


def _large_multigrid_grids(min_bus=15000):
    """The uneven multi-grid batch's grids of at least min_bus buses and their scenarios, made
    as the batch makes them (same sizes and seeds)."""
    from p3s_gb300.synthetic import make_grid, scenario_injections

    seed = 7
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(30), np.log(20000), 256)).astype(int)
    out = []
    for i, n in enumerate(sizes):
        if n >= min_bus:
            g = make_grid(int(n), seed=int(seed * 1000 + i), max_drop_pu=0.05)
            out.append((g, scenario_injections(g, 16, seed=int(seed * 1000 + i + 17))))
    return out


def test_large_grids_of_the_multigrid_batch():
    """Config-4 grids of 15,000 buses and more x 16 scenarios in ONE persistent launch."""
    from p3s_gb300.group import GpuGroup, GroupJob
    from p3s_gb300.solver import GpuSolver

    big = _large_multigrid_grids()
    assert len(big) >= 8 and max(g.n for g, _ in big) > 19000
    solvers = [GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq) for g, _ in big]
    grp = GpuGroup()
    jobs = [GroupJob(s, S, g.V0) for s, (g, S) in zip(solvers, big)]
    dbl = grp.solve(jobs, GpuSolver.params(precision="double"))
    mixed = grp.solve(jobs, GpuSolver.params(precision="mixed"))
    for (g, S), rd, rm in zip(big, dbl, mixed):
        osv = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
        ref = osv.solve_batch(S, g.V0)
        tight = osv.solve_batch(S, g.V0, tol=1e-12)
        assert ref["converged"].all()
        check_double(rd, ref, double_tol(g.n))
        check_mixed(rm, ref, tight, mismatch(g, rm["V"], S))


def test_largest_serving_topologies_through_the_server():
    """The serving pool's three largest topologies: a single solve, a 96-step chunk and a
    200-outage N-1 sweep each, admitted together into the serving loop (both precisions),
    against the oracle from the same warm start (the topology's converged base case); the
    stream launch's server gives the same results bit for bit."""
    from p3s_gb300 import contingency
    from p3s_gb300.serving import Request, Server, StreamServer, Topology
    from p3s_gb300.synthetic import make_grid

    sizes = _serving_sizes()
    picks = range(len(sizes) - 3, len(sizes))
    topos = [Topology(make_grid(int(sizes[i]), seed=500 + i, max_drop_pu=0.05)) for i in picks]
    assert [tp.n for tp in topos] == [26473, 42589, 49744]
    rq = np.random.default_rng(9)
    reqs = []
    for k, tp in enumerate(topos):
        g = tp.grid
        S1 = g.Sbus.copy()
        S1[g.pq] *= rq.uniform(0.8, 1.2, len(g.pq))
        reqs.append(Request(len(reqs), k, "single", 0.0, S1))
        Sc = np.repeat(g.Sbus[:, None], 96, axis=1)
        Sc[g.pq, :] *= rq.uniform(0.8, 1.2, (len(g.pq), 96))
        reqs.append(Request(len(reqs), k, "chunk", 0.0, np.ascontiguousarray(Sc)))
        outs = np.sort(rq.choice(len(g.f), 200, replace=False)).astype(np.int32)
        reqs.append(Request(len(reqs), k, "n1", 0.0, g.Sbus.copy(), outs))
    got = {}
    for prec in ("double", "mixed"):
        srv = Server(topos, precision=prec, contexts=2)
        got[prec] = srv.run(reqs, realtime=False)
        del srv
        stream = StreamServer(topos, precision=prec, capacity=64, arena_bytes=2 << 30, result_bytes=2 << 30)
        for a, b in zip(got[prec], stream.run(reqs, realtime=False)):
            assert np.array_equal(a.iterations, b.iterations) and np.array_equal(a.converged, b.converged)
            assert np.array_equal(np.isnan(a.V), np.isnan(b.V))
            assert np.array_equal(np.nan_to_num(a.V), np.nan_to_num(b.V))
            if a.served is not None:
                assert np.array_equal(a.served, b.served)
        del stream
    for q in reqs:
        tp = topos[q.topo]
        g = tp.grid
        osv = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
        if q.kind == "n1":
            groups = [[int(b)] for b in q.outages]
            batch = contingency.build_batch(g, groups=groups)
            lab, served, rb, _ = oisl.islands(g.n, g.f, g.t, batch.live, groups, g.ref, True, tp.prio)
            V0, pin = oisl.start_and_pins(tp.V_warm, served, rb, g.ref)
            Yx = batch.Yx_matrix
            mag, ang = np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx))
            ref = osv.solve_batch_contingency(mag, ang, q.S, V0, pin)
            tight = osv.solve_batch_contingency(mag, ang, q.S, V0, pin, tol=1e-12)
            for r in (ref, tight):
                r["V"] = np.where(served, r["V"], np.nan)
            S = np.repeat(q.S[:, None], len(groups), axis=1)
            tol_d = double_tol(g.n, TOL_V_N1)
        else:
            S = q.S[:, None] if q.S.ndim == 1 else q.S
            ref = osv.solve_batch(S, tp.V_warm)
            tight = osv.solve_batch(S, tp.V_warm, tol=1e-12)
            Yx, served, pin, tol_d = None, None, None, double_tol(g.n)
        assert ref["converged"].all()
        rd, rm = got["double"][q.rid], got["mixed"][q.rid]
        if served is not None:
            assert np.array_equal(rd.served, served) and np.array_equal(rm.served, served)
        check_double({"V": rd.V, "iterations": rd.iterations, "converged": rd.converged}, ref, tol_d)
        check_mixed({"V": rm.V, "iterations": rm.iterations, "converged": rm.converged}, ref, tight,
                    mismatch(g, rm.V, S, Yx, pin))


def test_flags_match_where_the_reference_falls_back_to_pivoting_lu(grid2000):
    """Cases on which the reference leaves its frozen pivot order for pivoting LU (nr_klu.cpp:
    610-652, 845-857; the oracle records each column's path): the 2,000-bus grid loaded 7.5x
    (near the nose: some cases converge on the frozen order, the rest are re-run on pivoting LU)
    and its full N-1 sweep loaded 6x. The device path has no pivoting LU; its convergence flags
    equal the reference's on every case (the fallback rescues none of these); where they converge,
    iterations and voltages as the other double-path bars. (A non-converged case reports the
    iteration at which its frozen-order factorization was rejected; the reference reports its
    pivoting retry's, up to max_iter.)"""
    import dataclasses

    from p3s_gb300 import contingency
    from p3s_gb300.cuda.nr_polar_solver import PolarNewtonSolverCUDA

    g = grid2000
    osv = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    S = np.ascontiguousarray(np.repeat(g.Sbus[:, None] * 7.5, 16, axis=1) * np.linspace(0.95, 1.05, 16)[None, :])
    ref = osv.solve_batch(S, g.V0)
    paths = osv.last_paths()
    assert (paths == 0).sum() >= 4 and (paths != 0).sum() >= 4
    gpu = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    check_converged(gpu.solve_batch(S, g.V0), ref, double_tol("2000x7.5"))
    gpu.precision = "mixed"
    assert np.array_equal(gpu.solve_batch(S, g.V0)["converged"], ref["converged"])

    g6 = dataclasses.replace(g, Sbus=g.Sbus * 6.0)
    batch = contingency.build_batch(g6)
    prio = np.zeros(g.n)
    prio[g.pv] = np.maximum(g.p_gen[g.pv], np.finfo(float).tiny)
    _, served, rb, _ = oisl.islands(g.n, g.f, g.t, batch.live, batch.groups, g.ref, True, prio)
    V0, pin = oisl.start_and_pins(g.V0, served, rb, g.ref)
    Yx = batch.Yx_matrix
    ref = osv.solve_batch_contingency(np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx)),
                                      g6.Sbus, V0, pin)
    ref["V"] = np.where(served, ref["V"], np.nan)
    paths = osv.last_paths()
    assert (paths != 0).sum() >= 5 and not ref["converged"][paths != 0].any()
    for prec in ("double", "mixed"):
        res = contingency.solve_contingencies(g6, reslack_islands=True, precision=prec, return_islands=False)
        assert np.array_equal(res.converged, ref["converged"]), prec
        if prec == "double":
            check_converged({"V": res.V, "iterations": res.iterations, "converged": res.converged}, ref,
                            double_tol("n1_2000x6", TOL_V_N1))
