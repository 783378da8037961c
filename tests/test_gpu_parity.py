"""GPU parity: the sm_103a path through the C ABI against the reference.

Bars (written next to each comparison): the plain double path reproduces the reference's
iteration counts and convergence flags exactly and its voltages to 1e-11; the mixed path
reaches the same solutions (1e-9) at <= 1e-8 mismatch; island labels and served masks are
bit-exact. Modelled on the reference's tests/cuda/test_lean_lu.py:126-326.
"""

import os

import numpy as np
import pytest

from oracle import cpu
from oracle.build import build_oracle
from p3s_gb300 import nr_klu
from p3s_gb300.cuda.nr_polar_solver import PolarNewtonSolverCUDA
from p3s_gb300.synthetic import grid_118, lanes, timeseries_injections

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_V = 1e-11  # plain double path vs the reference, per bus voltage (p.u.)


def setup_module(_):
    build_oracle()


def _g(name):
    return np.load(os.path.join(GOLDEN, name))


def _mismatch(d, V, S):
    """Infinity norm of the reference's mismatch F(V) per column (oracle debug_J's F)."""
    s = cpu.Solver(d.Yp, d.Yj, d.Yx, d.pv, d.pq)
    return np.array([np.abs(s.debug_J_at(S[:, c], V[:, c])["F"]).max() for c in range(V.shape[1])])


@pytest.mark.parametrize("name", ["golden_118.npz", "golden_2000.npz"])
def test_double_path_reproduces_reference(name):
    d = _g(name)
    r = nr_klu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch(d["S"], d["V0"])
    for tag in ("fast", "strict"):
        assert np.array_equal(r["converged"], d[f"cv_{tag}"])
        assert np.array_equal(r["iterations"], d[f"it_{tag}"])
        assert np.abs(r["V"] - d[f"V_{tag}"]).max() < TOL_V


def test_double_path_matches_oracle_on_a_2000_bus_batch(grid2000):
    S = timeseries_injections(grid2000, 192)
    ref = cpu.Solver(grid2000.Yp, grid2000.Yj, grid2000.Yx, grid2000.pv, grid2000.pq).solve_batch(S, grid2000.V0)
    gpu = PolarNewtonSolverCUDA(grid2000.Yp, grid2000.Yj, grid2000.Yx, grid2000.pv, grid2000.pq)
    r = gpu.solve_batch(S, grid2000.V0)
    assert r["converged"].all() and ref["converged"].all()
    assert np.array_equal(r["iterations"], ref["iterations"])
    assert np.abs(r["V"] - ref["V"]).max() < TOL_V
    assert gpu.last_stats["single_factorizations"] == 0 and gpu.last_stats["failed_on_gpu"] == 0
    # per-column start voltages take the same path as a shared one (bit-equal)
    r2 = gpu.solve_batch(S, np.ascontiguousarray(np.repeat(grid2000.V0[:, None], S.shape[1], axis=1)))
    assert np.array_equal(r2["V"], r["V"])


@pytest.mark.parametrize("ls", [1, 0])
def test_line_search_matches_reference_from_bad_starts(ls):
    d = _g("golden_118.npz")
    S = np.ascontiguousarray(np.repeat(d["Sbus"][:, None], d["V0_bad"].shape[1], axis=1))
    gpu = PolarNewtonSolverCUDA(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"])
    gpu.line_search = bool(ls)
    r = gpu.solve_batch(S, d["V0_bad"])
    ok = d[f"cvbad{ls}_strict"]
    assert 0 < ok.sum() < len(ok)
    assert np.array_equal(r["converged"], ok)
    assert np.array_equal(r["iterations"][ok], d[f"itbad{ls}_strict"][ok])
    assert np.abs(r["V"][:, ok] - d[f"Vbad{ls}_strict"][:, ok]).max() < 1e-10


@pytest.mark.parametrize("rule,switch", [("reference", 1e-3), ("gb300", 1e-3), ("gb300", 0.0)])
def test_mixed_precision_reaches_the_same_solution(grid2000, rule, switch):
    g = grid2000
    S = timeseries_injections(g, 128)
    ref = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
    gpu = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    double = gpu.solve_batch(S, g.V0)
    gpu.precision = "mixed"
    gpu.vote_rule = rule
    gpu.mixed_switch = switch
    mixed = gpu.solve_batch(S, g.V0)
    assert gpu.last_stats["single_factorizations"] > 0
    ok = ref["converged"]
    assert np.array_equal(mixed["converged"], ok)
    assert (_mismatch(g, mixed["V"][:, :16], S[:, :16]) <= 1e-8).all()
    # voltages: the oracle's own answer is only as exact as its last step (it stops anywhere
    # below tol), so the mixed result is held to 1e-9 against the oracle solved to
    # convergence (tol 1e-12), and to 1e-8 against the tol-1e-8 oracle
    ref_tight = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0, tol=1e-12)
    tight = ref_tight["converged"] & ok
    assert np.abs(mixed["V"][:, tight] - ref_tight["V"][:, tight]).max() < 1e-9
    assert np.abs(mixed["V"][:, ok] - ref["V"][:, ok]).max() < 1e-8
    assert (mixed["iterations"][ok] <= ref["iterations"][ok] + 2).all()
    # every float factorization rejected -> redone in double in the same step: the all-double run
    # (under the GB300 rule with the |J^-1| bound off, the all-double run to polish x tol)
    gpu._rcond_ratio_single = 1e30
    gpu.polish, gpu.vtol = 1e-3, 0.0
    rejected = gpu.solve_batch(S, g.V0)
    assert gpu.last_stats["single_rejected"] == gpu.last_stats["single_factorizations"] > 0
    if rule == "gb300":
        gpu.precision = "double"
        double = gpu.solve_batch(S, g.V0, tol=1e-8 * gpu.polish)
    assert np.array_equal(rejected["converged"], double["converged"])
    assert np.array_equal(rejected["iterations"], double["iterations"])
    assert np.array_equal(rejected["V"], double["V"])  # bit for bit: one mismatch for both paths


def test_non_finite_input_fails_only_its_own_column(grid118):
    S = timeseries_injections(grid118, 40)
    S[3, 7] = np.nan
    r = PolarNewtonSolverCUDA(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq).solve_batch(S, grid118.V0)
    expect = np.ones(40, dtype=bool)
    expect[7] = False
    assert np.array_equal(r["converged"], expect)
    assert np.isfinite(r["V"][:, expect]).all()


def test_rejected_factorization_is_reported_not_converged(grid118):
    S = timeseries_injections(grid118, 24)
    gpu = PolarNewtonSolverCUDA(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq)
    gpu._rcond_ratio = 1e30  # no factorization can pass the pivot check
    r = gpu.solve_batch(S, grid118.V0)
    assert not r["converged"].any()
    assert gpu.last_stats["failed_on_gpu"] == 24


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_invalid_start_voltage_raises_like_nr_klu(grid118, bad):
    V0 = grid118.V0.copy()
    V0[3] = complex(bad, 0.0)
    S = np.repeat(grid118.Sbus[:, None], 4, axis=1)
    with pytest.raises(RuntimeError, match="invalid initial voltage"):
        nr_klu.Solver(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq).solve_batch(S, V0)


def test_nan_admittance_is_never_reported_converged(grid118):
    Yx = grid118.Yx.copy()
    row = int(grid118.pq[0])
    k = [k for k in range(grid118.Yp[row], grid118.Yp[row + 1]) if grid118.Yj[k] == row][0]
    Yx[k] = complex(np.nan, 0.0)
    S = np.ascontiguousarray(np.repeat(grid118.Sbus[:, None], 4, axis=1))
    # nr_klu surface: the solver builds, every column ends not converged (nr_klu semantics)
    r = nr_klu.Solver(grid118.Yp, grid118.Yj, Yx, grid118.pv, grid118.pq).solve_batch(S, grid118.V0)
    assert not r["converged"].any()
    # PolarNewtonSolverCUDA surface: refuses the grid at construction (nr_polar_solver.py:422-426)
    with pytest.raises(RuntimeError, match="flat start"):
        PolarNewtonSolverCUDA(grid118.Yp, grid118.Yj, Yx, grid118.pv, grid118.pq)
    # a NaN admittance in one case of a batch fails only that batch's NaN cases
    gpu = PolarNewtonSolverCUDA(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq)
    r = gpu.solve_batch_contingency_cx(np.repeat(Yx[:, None], 4, axis=1), grid118.Sbus,
                                       np.repeat(grid118.V0[:, None], 4, axis=1), np.zeros((118, 4), np.uint8))
    assert not r["converged"].any()


def test_update_Y_equals_rebuilding_the_solver(grid118):
    S = timeseries_injections(grid118, 16)
    # new branch parameters (every branch's stamp scaled by 1 +- 3%), same pattern
    st = grid118.stamp * (1.0 + 0.03 * np.random.default_rng(4).standard_normal(grid118.n_branch))[:, None]
    Yx2 = np.zeros(grid118.nnz, dtype=complex)
    np.add.at(Yx2, grid118.stamp_pos.ravel(), st.ravel())
    gpu = PolarNewtonSolverCUDA(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq)
    before = gpu.solve_batch(S, grid118.V0)["V"]
    gpu.update_Y(Yx2)
    after = gpu.solve_batch(S, grid118.V0)
    fresh = PolarNewtonSolverCUDA(grid118.Yp, grid118.Yj, Yx2, grid118.pv, grid118.pq).solve_batch(S, grid118.V0)
    assert after["converged"].all()
    assert np.array_equal(after["V"], fresh["V"])
    assert np.abs(after["V"] - before).max() > 1e-6
    with pytest.raises(ValueError):
        gpu.update_Y(Yx2[:-1])


def test_debug_J_matches_reference():
    d = _g("golden_118.npz")
    j = nr_klu.debug_J(d["Yp"], d["Yj"], d["Yx"], d["Sbus"], d["V0"], d["pv"], d["pq"])
    assert np.array_equal(j["Jp"], d["Jp"]) and np.array_equal(j["Ji"], d["Ji"])
    assert np.abs(j["Jx"] - d["Jx"]).max() < 1e-10


def test_solve_single_and_solve(grid118):
    ref = cpu.solve_single(grid118.Yp, grid118.Yj, grid118.Yx, grid118.Sbus, grid118.V0, grid118.pv, grid118.pq)
    r = nr_klu.solve_single(grid118.Yp, grid118.Yj, grid118.Yx, grid118.Sbus, grid118.V0, grid118.pv, grid118.pq)
    assert set(r) >= {"V", "iterations", "converged", "t_setup_ms", "t_solve_ms", "t_assemble_ms", "profiled"}
    assert r["iterations"] == ref["iterations"] and r["converged"]
    assert np.abs(r["V"] - ref["V"]).max() < TOL_V


def test_results_do_not_depend_on_the_batch_mix(grid2000):
    """Continuous batching: a case gives the same bits alone, in a batch, and in a
    differently composed batch (slots are independent)."""
    g = grid2000
    S = timeseries_injections(g, 300)
    gpu = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    full = gpu.solve_batch(S, g.V0)
    idx = np.random.default_rng(3).permutation(300)[:37]
    part = gpu.solve_batch(np.ascontiguousarray(S[:, idx]), g.V0)
    assert np.array_equal(part["V"], full["V"][:, idx])
    one = gpu.solve_batch(np.ascontiguousarray(S[:, idx[:1]]), g.V0)
    assert np.array_equal(one["V"][:, 0], full["V"][:, idx[0]])


def test_warm_start_lanes_match_the_oracle_replay(grid2000):
    g = grid2000
    S = timeseries_injections(g, 120)
    off = lanes(120, 16)
    ref = cpu.solve_lanes(cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq), S, g.V0, off)
    gpu = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    r = gpu.solve_timeseries_lanes(S, g.V0, off)
    assert r["converged"].all() and ref["converged"].all()
    assert np.array_equal(r["iterations"], ref["iterations"])
    assert np.abs(r["V"] - ref["V"]).max() < TOL_V
    assert r["iterations"].mean() < 6  # warm starts pay off


def test_contingency_stamps_equal_dense_and_reference():
    d = _g("golden_n1_118.npz")
    L = d["pin"].shape[1]
    Yx = np.repeat(d["Yx"][:, None], L, axis=1)
    rows, cols, vals = [], [], []
    for c in range(1, L):
        b = c - 1
        np.subtract.at(Yx[:, c], d["stamp_pos"][b], d["stamp"][b])
        rows.append(d["stamp_pos"][b])
        cols.append(np.full(4, c))
        vals.append(d["stamp"][b])
    import scipy.sparse as sp

    stamp = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(len(d["Yx"]), L)).tocsc()
    gpu = PolarNewtonSolverCUDA(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"])
    dense = gpu.solve_batch_contingency_cx(Yx, d["Sbus"], d["V0n1"], d["pin"])
    st = gpu.solve_batch_contingency_stamp(stamp, d["Sbus"], d["V0n1"], d["pin"])
    polar = gpu.solve_batch_contingency(np.abs(Yx), np.angle(Yx), d["Sbus"], d["V0n1"], d["pin"])
    ok = d["cv_strict"]
    assert np.array_equal(dense["converged"], ok) and ok.any()
    assert np.array_equal(st["V"], dense["V"])
    assert np.array_equal(st["iterations"], d["it_strict"]) or np.array_equal(st["iterations"][ok],
                                                                               d["it_strict"][ok])
    assert np.abs(dense["V"][:, ok] - d["V_strict"][:, ok]).max() < 1e-10
    assert np.abs(polar["V"][:, ok] - d["V_strict"][:, ok]).max() < 1e-10
    # the nr_klu surface takes magnitude / angle
    nk = nr_klu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch_contingency(
        np.abs(Yx), np.angle(Yx), d["Sbus"], d["V0n1"], d["pin"])
    assert np.array_equal(nk["converged"], ok)


def test_islands_match_reference_bit_exact():
    from p3s_gb300 import contingency

    d = _g("golden_n1_118.npz")
    g = grid_118()
    assert np.array_equal(g.Yx, d["Yx"])
    batch = contingency.build_batch(g)
    prio = np.zeros(g.n)
    prio[g.pv] = g.p_gen[g.pv]
    lab, sv, rb, ni = contingency.islands(batch, True, prio)
    assert lab.dtype == np.int32
    assert np.array_equal(lab, d["labels"]) and np.array_equal(sv, d["served"])
    assert np.array_equal(rb, d["ref_bus"]) and np.array_equal(ni, d["n_islands"])
    lab0, sv0, rb0, _ = contingency.islands(batch, False, prio)
    assert np.array_equal(lab0, d["labels"]) and (sv0 <= sv).all() and (~sv0).sum() > (~sv).sum()


def test_contingency_driver_matches_reference():
    from p3s_gb300 import contingency

    d = _g("golden_n1_118.npz")
    g = grid_118()
    res = contingency.solve_contingencies(g, reslack_islands=True)
    assert np.array_equal(res.served, d["served"])
    ok = d["cv_strict"]
    assert np.array_equal(res.converged, ok)
    assert np.isnan(res.V[~res.served]).all() and np.isfinite(res.V[:, ok][res.served[:, ok]]).all()
    Vs = np.where(d["served"], d["V_strict"], np.nan)
    assert np.nanmax(np.abs(res.V[:, ok] - Vs[:, ok])) < 1e-10
    mixed = contingency.solve_contingencies(g, reslack_islands=True, precision="mixed")
    assert np.array_equal(mixed.converged, ok) and np.array_equal(mixed.served, d["served"])
    assert np.nanmax(np.abs(mixed.V[:, ok] - Vs[:, ok])) < 1e-8
    # against the oracle solved to convergence (tol 1e-12)
    L = d["pin"].shape[1]
    Yx = np.repeat(d["Yx"][:, None], L, axis=1)
    for c in range(1, L):
        np.subtract.at(Yx[:, c], d["stamp_pos"][c - 1], d["stamp"][c - 1])
    tight = cpu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch_contingency(
        np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx)), d["Sbus"], d["V0n1"], d["pin"],
        tol=1e-12)
    ok2 = ok & tight["converged"]
    Vt = np.where(d["served"], tight["V"], np.nan)
    assert np.nanmax(np.abs(mixed.V[:, ok2] - Vt[:, ok2])) < 1e-9


def test_integer_pipe_conversions_match_ieee():
    """The kernels' float <-> double helpers: float -> double exact; double -> float within
    one float ulp of the IEEE cast (it truncates), zero / infinity / NaN preserved."""
    import ctypes as C

    from p3s_gb300 import _lib

    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(4000) * 10.0 ** rng.integers(-30, 30, 4000),
                        [0.0, -0.0, 1.0, -1.0, 3.4e38, 1e39, -1e39, 1e-39, np.inf, -np.inf, np.nan]])
    x = np.ascontiguousarray(x)
    d2f = np.empty(len(x), np.float32)
    f2d = np.empty(len(x), np.float64)
    small = np.empty(len(x), np.float32)
    fp = C.POINTER(C.c_float)
    rc = _lib.load().gbpf_selftest_conversions(_lib.d(x), len(x), d2f.ctypes.data_as(fp), _lib.d(f2d),
                                               small.ctypes.data_as(fp))
    assert rc == 0, _lib.last_error()
    ref = x.astype(np.float32)
    normal = np.isfinite(ref) & (np.abs(ref) >= np.finfo(np.float32).tiny)
    ulp = np.spacing(np.abs(ref[normal]).astype(np.float32))
    assert (np.abs(d2f[normal].astype(np.float64) - ref[normal].astype(np.float64)) <= ulp).all()
    assert (np.abs(d2f[normal]) <= np.abs(ref[normal])).all()  # toward zero
    assert np.array_equal(f2d[normal], d2f[normal].astype(np.float64))  # exact widening
    assert np.isnan(d2f[-1]) and np.isinf(d2f[-3]) and d2f[-3] > 0 and np.isinf(d2f[-2]) and d2f[-2] < 0
    assert d2f[x == 0.0].tolist() == [0.0, 0.0]
    # the float Jacobian's short conversion: the same bits wherever it is used (|x| < 2^128)
    inr = np.isfinite(x) & (np.abs(x) < 2.0 ** 128)
    assert np.array_equal(small[inr].view(np.uint32), d2f[inr].view(np.uint32))


def test_own_double_numerics_within_an_ulp():
    """The kernels' own double-precision helpers against exact references: the Newton-refined
    reciprocal (a float seed and two Newton-Raphson steps) within 2 ulp of IEEE 1/x over the
    voltage-magnitude range and beyond, and the small-angle Maclaurin sine / cosine used to
    rotate phasors within 1 ulp of numpy's (and of CUDA's sincos) over |d| < 1/4."""
    from p3s_gb300 import _lib

    rng = np.random.default_rng(3)
    x = np.concatenate([10.0 ** rng.uniform(-6, 6, 20000), rng.uniform(0.5, 1.5, 20000),
                        [1e-6, 0.9, 1.0, 1.04, 10.0, 1e6]])
    d = np.concatenate([rng.uniform(-0.25, 0.25, 20000) * 2.0 ** -rng.integers(0, 40, 20000),
                        [0.0, -0.0, 2.0 ** -14, -(2.0 ** -6), 0.2499999]])
    inp = np.ascontiguousarray(np.concatenate([x, d]))
    outs = [np.empty(len(inp)) for _ in range(5)]
    ph = np.array([np.cos(0.7), np.sin(0.7)])
    rot = np.empty((len(inp), 4))
    rc = _lib.load().gbpf_selftest_math(_lib.d(inp), len(inp), *[_lib.d(o) for o in outs], _lib.d(ph), _lib.d(rot))
    assert rc == 0, _lib.last_error()
    recip, s_small, c_small, s_ref, c_ref = outs
    nx = len(x)
    want = 1.0 / x
    assert (np.abs(recip[:nx] - want) <= 2 * np.spacing(want)).all()
    dd = inp[nx:]
    for got, cuda, exact in ((s_small[nx:], s_ref[nx:], np.sin(dd)), (c_small[nx:], c_ref[nx:], np.cos(dd))):
        ulp = np.spacing(np.abs(exact))
        assert (np.abs(got - exact) <= ulp).all()
        assert (np.abs(got - cuda) <= 2 * ulp).all()
    assert s_small[nx + 20000] == 0.0 and c_small[nx + 20000] == 1.0
    # the voltage update's rotation of a committed phasor by the increment d against the rotation
    # of the same double phasor in extended precision: within 2 ulp
    L = np.longdouble
    c0, s0 = L(ph[0]), L(ph[1])
    dl = dd.astype(L)
    want_c = (c0 * np.cos(dl) - s0 * np.sin(dl)).astype(np.float64)
    want_s = (s0 * np.cos(dl) + c0 * np.sin(dl)).astype(np.float64)
    assert (np.abs(rot[nx:, 0] - want_c) <= 2 * np.spacing(np.abs(want_c))).all()
    assert (np.abs(rot[nx:, 1] - want_s) <= 2 * np.spacing(np.abs(want_s))).all()
    # after a float step at a PQ bus the increment is formed in float from truncated float
    # copies (each within 2^-23): within 2^-20 |d| (plus the double addition's rounding) of the
    # exact rotation
    bound = 2.0 ** -20 * np.abs(dd) + 2 * np.spacing(1.0)
    assert (np.abs(rot[nx:, 2] - want_c) <= bound).all() and (np.abs(rot[nx:, 3] - want_s) <= bound).all()


def test_n1_sweep_of_the_2000_bus_grid(grid2000):
    """The full N-1 sweep (base case + every single-branch outage): islands, served masks and
    references bit-exact against the restated reference islanding for all 3,001 cases; the
    solves of a sample (every islanded case plus random ones) against the oracle."""
    from oracle import islands as oisl
    from p3s_gb300 import contingency

    g = grid2000
    batch = contingency.build_batch(g)
    assert len(batch.groups) == g.n_branch + 1
    prio = np.zeros(g.n)
    prio[g.pv] = g.p_gen[g.pv]
    lab, sv, rb, ni = contingency.islands(batch, True, prio)
    olab, osv, orb, oni = oisl.islands(g.n, g.f, g.t, batch.live, batch.groups, g.ref, True, prio)
    assert np.array_equal(lab, olab) and np.array_equal(sv, osv)
    assert np.array_equal(rb, orb) and np.array_equal(ni, oni)
    split = np.nonzero(ni > 1)[0]
    assert len(split) > 0
    rng = np.random.default_rng(3)
    pick = np.union1d(split[:48], rng.choice(len(batch.groups), 48, replace=False))
    groups = [batch.groups[c] for c in pick]
    sub = contingency.build_batch(g, groups=groups)
    s_lab, s_sv, s_rb, _ = contingency.islands(sub, True, prio)
    V0, pin = contingency.start_and_pins(sub, g.V0, s_sv, s_rb)
    Yx = sub.Yx_matrix
    osolver = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    ref = osolver.solve_batch_contingency(np.abs(Yx), np.angle(Yx), g.Sbus, V0, pin)
    ok = ref["converged"]
    assert ok.all()
    res = contingency.solve_contingencies(g, reslack_islands=True, groups=groups)
    assert np.array_equal(res.served, s_sv) and np.array_equal(res.converged, ok)
    assert np.array_equal(res.labels, s_lab) and np.array_equal(res.ref_bus, s_rb)
    # the served mask comes from the launch's own islanding (no separate islanding call)
    res2 = contingency.solve_contingencies(g, reslack_islands=True, groups=groups, return_islands=False)
    assert res2.labels is None and res2.served.dtype == bool and np.array_equal(res2.served, s_sv)
    assert np.array_equal(np.isnan(res2.V), ~s_sv) and np.array_equal(res2.iterations, res.iterations)
    assert np.array_equal(res.iterations, ref["iterations"])
    Vs = np.where(s_sv, ref["V"], np.nan)
    assert np.nanmax(np.abs(res.V - Vs)) < 1e-10  # the oracle rebuilds each Ybus from |Y| and angle
    mixed = contingency.solve_contingencies(g, reslack_islands=True, groups=groups, precision="mixed")
    tight = osolver.solve_batch_contingency(np.abs(Yx), np.angle(Yx), g.Sbus, V0, pin, tol=1e-12)
    assert np.array_equal(mixed.converged, ok) and tight["converged"].all()
    assert np.nanmax(np.abs(mixed.V - np.where(s_sv, tight["V"], np.nan))) < 1e-9


def test_results_do_not_depend_on_the_cta_shape(grid2000):
    """Every CTA shape and every factorization schedule (chain caps: chains cut finer,
    coarser or never) runs the same arithmetic per case: the batch-size rule, a pinned shape,
    a chain cap and the autotuner change only the speed, never a bit of the result."""
    from p3s_gb300.autotune import tune, tune_lanes
    from p3s_gb300.solver import GpuSolver

    g = grid2000
    S = timeseries_injections(g, 96)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    off = lanes(96, 96)
    assert s.shape(1) == (1024, 1) and s.shape(8760) == (512, 32)
    for prec in ("double", "mixed"):
        p = GpuSolver.params(precision=prec)
        base = s.solve_lanes(S, g.V0, off, p)
        for nt, slots in ((1024, 4), (512, 8), (256, 16), (512, 32)):
            s.set_shape(96, nt, slots)
            assert s.shape(96) == (nt, slots)
            r = s.solve_lanes(S, g.V0, off, p)
            assert s.stats["threads_per_cta"] == nt and s.stats["cases_per_cta"] == slots
            assert np.array_equal(r["V"], base["V"]) and np.array_equal(r["iterations"], base["iterations"])
        s.set_shape(96, 0, 0)
        for cap in (0.0, 0.25, 2.0):
            s.set_chain_cap(cap)
            r = s.solve_lanes(S, g.V0, off, p)
            assert np.array_equal(r["V"], base["V"]) and np.array_equal(r["iterations"], base["iterations"])
        s.set_chain_cap(1.0)
    choice, timings = tune_lanes(s, S, g.V0, off, GpuSolver.params(precision="mixed"),
                                 candidates=((1024, 2), (512, 4)), reps=1)
    assert s.shape(96) == choice and set(timings) == {(1024, 2), (512, 4)}
    p = GpuSolver.params(precision="mixed")
    choice, timings = tune(s, 96, lambda: s.solve_lanes(S, g.V0, off, p), candidates=((512, 4),),
                           chain_caps=(1.0, 0.0), reps=1)
    assert set(timings) == {(512, 4, 1.0), (512, 4, 0.0)} and s.chain_cap == choice[2]
    assert s.shape(96) == choice[:2]


def test_uneven_grids_in_one_launch_match_their_own_solves():
    """Grids of uneven size in ONE persistent launch (a group): every result equals the grid's
    own single-topology solve bit for bit, and the double path matches the oracle."""
    from p3s_gb300.group import GpuGroup, GroupJob
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.synthetic import make_grid, scenario_injections

    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(30), np.log(3000), 12)).astype(int)
    grids = [make_grid(int(n), seed=100 + i) for i, n in enumerate(sizes)]
    scen = [scenario_injections(g, 16, seed=200 + i) for i, g in enumerate(grids)]
    solvers = [GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq) for g in grids]
    grp = GpuGroup()
    for prec in ("double", "mixed"):
        p = GpuSolver.params(precision=prec)
        res = grp.solve([GroupJob(s, S, g.V0) for s, S, g in zip(solvers, scen, grids)], p)
        assert grp.stats["single_factorizations" if prec == "mixed" else "double_factorizations"] > 0
        for s, S, g, r in zip(solvers, scen, grids, res):
            alone = s.solve_batch(S, g.V0, p)
            assert np.array_equal(r["V"], alone["V"]) and np.array_equal(r["iterations"], alone["iterations"])
            assert np.array_equal(r["converged"], alone["converged"]) and r["converged"].all()
        if prec == "double":
            for i in (0, len(grids) // 2, len(grids) - 1):
                g = grids[i]
                ref = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(scen[i], g.V0)
                assert np.array_equal(res[i]["iterations"], ref["iterations"])
                assert np.abs(res[i]["V"] - ref["V"]).max() < TOL_V


def test_async_slots_overlap_and_equal_the_synchronous_call(grid2000):
    from p3s_gb300.solver import GpuSolver, pinned_empty

    g = grid2000
    T = 256
    S = timeseries_injections(g, T)
    off = lanes(T, 64)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    p = GpuSolver.params(precision="mixed")
    ref = s.solve_lanes(S, g.V0, off, p)
    outs = []
    for slot in range(2):
        Sh = pinned_empty(S.shape, np.complex128)
        Sh[...] = S
        out = (pinned_empty((g.n, T), np.complex128), pinned_empty((T,), np.int32), pinned_empty((T,), np.uint8))
        s.solve_lanes_async(slot, Sh, g.V0, off, p, out)
        outs.append(out)
    with pytest.raises(RuntimeError, match="still in flight"):
        s.solve_lanes_async(0, S, g.V0, off, p, outs[0])
    for slot in range(2):
        s.wait(slot)
        V, it, cv = outs[slot]
        assert np.array_equal(V, ref["V"]) and np.array_equal(it, ref["iterations"])
        assert np.array_equal(cv.astype(bool), ref["converged"])
    with pytest.raises(RuntimeError, match="nothing in flight"):
        s.wait(0)


def test_chord_polish_steps_keep_the_solution(grid2000):
    """Polish steps that reuse the previous float factors (chord_tol) reach the same converged
    voltages as refactoring every step: both within 1e-9 of the oracle solved to convergence,
    every step counted once as a factorization or a chord step."""
    from p3s_gb300.solver import GpuSolver

    g = grid2000
    S = timeseries_injections(g, 256)
    ref = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0, tol=1e-12)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    off = lanes(256, 256)
    out = {}
    for ct in (0.0, 1e-8, 1e-6):
        r = s.solve_lanes(S, g.V0, off, GpuSolver.params(precision="mixed", chord_tol=ct))
        st = s.stats
        assert r["converged"].all()
        steps = int(r["iterations"].sum())
        # every step one float factorization, chord step, first step with the shared start's
        # factors or double factorization (a rejected float factorization is redone in double
        # in the same step)
        assert (st["single_factorizations"] + st["double_factorizations"] + st["chord_steps"] + st["first_steps"]
                == steps + st["single_rejected"])
        assert st["first_steps"] == 256  # every case starts from the shared V0
        assert (st["chord_steps"] == 0) == (ct == 0.0)
        assert np.abs(r["V"] - ref["V"]).max() < 1e-9  # tolerance: mixed path vs converged oracle
        assert (_mismatch(g, r["V"][:, :8], S[:, :8]) <= 1e-8).all()
        out[ct] = r
    assert (out[1e-8]["iterations"] <= out[0.0]["iterations"] + 1).all()
    # the lazy Jacobian (left out where no factorization is expected, built later if one
    # follows after all) changes nothing: bit for bit the run that builds every Jacobian
    lazy, st_lazy = out[1e-8], None
    r = s.solve_lanes(S, g.V0, off, GpuSolver.params(precision="mixed", chord_tol=1e-8))
    st_lazy = s.stats
    eager = s.solve_lanes(S, g.V0, off, GpuSolver.params(precision="mixed", chord_tol=1e-8, eager_jacobian=True))
    assert st_lazy["lazy_jacobians"] > 0 and s.stats["lazy_jacobians"] == 0
    assert np.array_equal(r["V"], eager["V"]) and np.array_equal(r["iterations"], eager["iterations"])
    assert np.array_equal(lazy["V"], eager["V"])


def test_shared_start_equals_each_case_starting_on_its_own(grid2000):
    """Cases that all start from one V0 take their first step with that start's injections and
    factors, computed once per launch (stats["first_steps"]); the result is, bit for bit, what
    every case gets from its own copy of V0 (its own first evaluation and factorization)."""
    from p3s_gb300.solver import GpuSolver

    g = grid2000
    T = 64
    S = timeseries_injections(g, T)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    own_V0 = np.ascontiguousarray(np.repeat(g.V0[:, None], T, axis=1))
    for prec in ("mixed", "double"):
        p = GpuSolver.params(precision=prec)
        shared = s.solve_batch(S, g.V0, p)
        assert s.stats["first_steps"] == T
        own = s.solve_batch(S, own_V0, p)
        assert s.stats["first_steps"] == 0
        assert np.array_equal(shared["iterations"], own["iterations"])
        assert np.array_equal(shared["V"], own["V"])
        assert shared["converged"].all()


def test_per_result_accuracy_bound_covers_the_distance_to_the_converged_oracle(grid2000):
    """Every mixed result carries its final mismatch and |J^-1| x mismatch (``error_bound``); the
    bound covers the result's distance from the oracle solved to convergence (tol 1e-12), up to
    that oracle's own bound, and last_stats states the largest one."""
    g = grid2000
    S = timeseries_injections(g, 96)
    tight = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0, tol=1e-12)
    gpu = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    gpu.precision = "mixed"
    r = gpu.solve_batch(S, g.V0)
    assert r["converged"].all() and tight["converged"].all()
    jinv = gpu.last_stats["jinv_norm"]
    assert jinv > 1.0 and (r["mismatch"] <= 1e-8).all()
    assert np.array_equal(r["error_bound"], r["mismatch"] * jinv)
    dist = np.abs(r["V"] - tight["V"]).max(axis=0)
    assert (dist <= r["error_bound"] + jinv * 1e-12).all()
    assert gpu.last_stats["error_bound"] == r["error_bound"].max() < 1e-7
    # the double path records its own
    gpu.precision = "double"
    rd = gpu.solve_batch(S, g.V0)
    assert (rd["mismatch"] < 1e-8).all() and gpu.last_stats["max_mismatch"] == rd["mismatch"].max()
