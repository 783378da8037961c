"""CPU oracle pinned against the reference: golden fixtures produced by the reference's own
nr_klu.cpp (tests/golden/make_golden.py), and -- where the reference build exists -- a
bit-for-bit comparison on fresh inputs. Mirrors the reference's guards
(tests/cpp/test_cpp_threading_guards.py, p3s/cpp/tests/test_batch.py)."""

import os

import numpy as np
import pytest

from oracle import cpu
from oracle import islands as oi
from oracle.build import build_oracle, load_reference

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def setup_module(_):
    build_oracle()


def _g(name):
    return np.load(os.path.join(GOLDEN, name))


def test_oracle_matches_reference_golden_118():
    d = _g("golden_118.npz")
    r = cpu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch(d["S"], d["V0"])
    for tag, tol in (("strict", 1e-12), ("fast", 1e-11)):
        assert np.array_equal(r["iterations"], d[f"it_{tag}"])
        assert np.array_equal(r["converged"], d[f"cv_{tag}"])
        assert np.abs(r["V"] - d[f"V_{tag}"]).max() < tol


def test_oracle_matches_reference_golden_2000():
    d = _g("golden_2000.npz")
    r = cpu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch(d["S"], d["V0"])
    assert r["converged"].all()
    for tag, tol in (("strict", 1e-12), ("fast", 1e-11)):
        assert np.array_equal(r["iterations"], d[f"it_{tag}"])
        assert np.abs(r["V"] - d[f"V_{tag}"]).max() < tol


@pytest.mark.parametrize("ls", [1, 0])
def test_oracle_line_search_decisions_match_reference(ls):
    d = _g("golden_118.npz")
    S = np.ascontiguousarray(np.repeat(d["Sbus"][:, None], d["V0_bad"].shape[1], axis=1))
    r = cpu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch(S, d["V0_bad"], line_search=bool(ls))
    ok = d[f"cvbad{ls}_strict"]
    assert 0 < ok.sum() < len(ok)
    for tag in ("strict", "fast"):
        assert np.array_equal(r["converged"], d[f"cvbad{ls}_{tag}"])
        assert np.array_equal(r["iterations"][ok], d[f"itbad{ls}_{tag}"][ok])
    assert np.abs(r["V"][:, ok] - d[f"Vbad{ls}_strict"][:, ok]).max() < 1e-12
    # damping changes the outcome of this sweep (the reference test's own precondition)
    assert not np.array_equal(d["itbad1_strict"], d["itbad0_strict"])


def test_oracle_jacobian_matches_reference():
    d = _g("golden_118.npz")
    j = cpu.debug_J(d["Yp"], d["Yj"], d["Yx"], d["Sbus"], d["V0"], d["pv"], d["pq"])
    assert np.array_equal(j["Jp"], d["Jp"]) and np.array_equal(j["Ji"], d["Ji"])
    assert np.abs(j["Jx"] - d["Jx"]).max() < 1e-12


def test_oracle_contingency_matches_reference():
    d = _g("golden_n1_118.npz")
    nnz = len(d["Yj"])
    L = d["pin"].shape[1]
    Yx = np.repeat(d["Yx"][:, None], L, axis=1)
    for c in range(1, L):  # case c >= 1 outages branch c - 1
        b = c - 1
        np.subtract.at(Yx[:, c], d["stamp_pos"][b], d["stamp"][b])
    assert Yx.shape == (nnz, L)
    r = cpu.Solver(d["Yp"], d["Yj"], d["Yx"], d["pv"], d["pq"]).solve_batch_contingency(
        np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx)), d["Sbus"], d["V0n1"], d["pin"])
    ok = d["cv_strict"]
    assert ok.sum() > 0.9 * L
    assert np.array_equal(r["converged"], ok)
    assert np.array_equal(r["iterations"][ok], d["it_strict"][ok])
    assert np.abs(r["V"][:, ok] - d["V_strict"][:, ok]).max() < 1e-11


def test_oracle_islands_match_reference():
    d = _g("golden_n1_118.npz")
    live = (d["stamp"][:, 1] != 0) | (d["stamp"][:, 2] != 0)
    groups = [[]] + [[b] for b in range(len(d["f"]))]
    prio = np.zeros(len(d["Yp"]) - 1)
    prio[d["pv"]] = d["p_gen"][d["pv"]]
    lab, sv, rb, ni = oi.islands(len(d["Yp"]) - 1, d["f"], d["t"], live, groups, d["ref"], True, prio)
    assert np.array_equal(lab, d["labels"]) and np.array_equal(sv, d["served"])
    assert np.array_equal(rb, d["ref_bus"]) and np.array_equal(ni, d["n_islands"])


def test_oracle_bit_equal_to_reference_build(grid118):
    strict = load_reference("strict")
    if strict is None:
        pytest.skip("reference build (oracle/_ref) not available")
    from p3s_gb300.synthetic import grid_118, timeseries_injections

    for seed in (1, 2):
        g = grid_118(seed)
        S = timeseries_injections(g, 12, seed=seed)
        a = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
        b = strict.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
        assert np.array_equal(a["V"], b["V"]) and np.array_equal(a["iterations"], b["iterations"])


def test_oracle_thread_invariance(grid118):
    from p3s_gb300.synthetic import timeseries_injections

    S = timeseries_injections(grid118, 24)
    s = cpu.Solver(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq)
    r1 = s.solve_batch(S, grid118.V0, n_threads=1)
    r4 = s.solve_batch(S, grid118.V0, n_threads=4)
    assert np.array_equal(r1["V"], r4["V"]) and np.array_equal(r1["iterations"], r4["iterations"])


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_oracle_rejects_non_finite_start(grid118, bad):
    V0 = grid118.V0.copy()
    V0[3] = complex(bad, 0.0)
    S = np.repeat(grid118.Sbus[:, None], 4, axis=1)
    with pytest.raises(RuntimeError, match="invalid initial voltage"):
        cpu.Solver(grid118.Yp, grid118.Yj, grid118.Yx, grid118.pv, grid118.pq).solve_batch(S, V0)


def test_oracle_nan_admittance_never_converges(grid118):
    Yx = grid118.Yx.copy()
    row = int(grid118.pq[0])
    k = [k for k in range(grid118.Yp[row], grid118.Yp[row + 1]) if grid118.Yj[k] == row][0]
    Yx[k] = complex(np.nan, 0.0)
    S = np.repeat(grid118.Sbus[:, None], 4, axis=1)
    r = cpu.Solver(grid118.Yp, grid118.Yj, Yx, grid118.pv, grid118.pq).solve_batch(S, grid118.V0)
    assert not r["converged"].any()
