"""Generate the golden fixtures from the REFERENCE's own solver.

Runs the reference's p3s/cpp/nr_klu.cpp, compiled by oracle/build.py (both the release-flag
build and the strict-IEEE build), on seeded synthetic inputs and stores inputs and results:

* golden_118.npz   -- 118-bus grid, 32 hourly columns (flat start) and 48 scrambled-angle
                      starts solved with and without line search;
* golden_2000.npz  -- 2,000-bus grid, 4 hourly columns;
* golden_n1_118.npz -- 118-bus N-1 (intact + every branch outage, re-slacked islands):
                      island labels / served masks / reference buses from the reference's own
                      ContingencyCaseGenerator._components_after_outage / _resolve_references
                      (p3s/contingency/case_generator.py:355-430, imported with its pandapower
                      dependencies stubbed out and generator impedance z = 1 / P, so "lowest
                      impedance" = "largest scheduled P"), and the reference's
                      solve_batch_contingency results.

Usage (needs the reference checkout and pybind11): python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "parallel-pandapower-solver_gb300"), ROOT]

from oracle import build as ob  # noqa: E402
from oracle import islands as oi  # noqa: E402
from p3s_gb300 import contingency  # noqa: E402
from p3s_gb300.synthetic import grid_118, grid_2000, timeseries_injections  # noqa: E402


def grid_arrays(g):
    return dict(Yp=g.Yp, Yj=g.Yj, Yx=g.Yx, pv=g.pv, pq=g.pq, ref=g.ref, Sbus=g.Sbus, V0=g.V0, f=g.f, t=g.t,
                stamp=g.stamp, stamp_pos=g.stamp_pos, p_gen=g.p_gen)


def reference_islands(g, batch, prio):
    """Island labels / served / reference bus of every case from the reference's own code."""
    import types

    ref_root = os.path.dirname(os.path.dirname(ob.REF_CPP))  # the reference checkout
    if ref_root not in sys.path:
        sys.path.append(ref_root)
    gt = types.ModuleType("p3s.contingency.ground_truth")
    gt.enumerate_contingencies = gt.generator_z_pu = None
    npf = types.ModuleType("p3s.NewtonPowerflow")
    npf.NewtonPowerflow = object
    sys.modules.setdefault("p3s.contingency.ground_truth", gt)
    sys.modules.setdefault("p3s.NewtonPowerflow", npf)
    from p3s.contingency.case_generator import ContingencyCaseGenerator

    gen = ContingencyCaseGenerator.__new__(ContingencyCaseGenerator)
    gen.n_bus = g.n
    gen._br_from = np.asarray(g.f, dtype=np.int64)
    gen._br_to = np.asarray(g.t, dtype=np.int64)
    gen._br_live = np.asarray(batch.live, dtype=bool)
    gen.ref = np.asarray(g.ref, dtype=np.int64)
    gen.reslack_islands = True
    gens = np.nonzero(prio > 0)[0]
    z = 1.0 / prio[gens]
    zs = np.sort(z)
    assert not np.any(np.isclose(zs[1:], zs[:-1])), "tied generator ranks: pick another seed"
    gen._gen_z = {int(b): float(v) for b, v in zip(gens, z)}
    L = len(batch.groups)
    labels = np.empty((g.n, L), dtype=np.int32)
    served = np.empty((g.n, L), dtype=bool)
    ref_bus = np.empty((g.n, L), dtype=np.int32)
    nis = np.empty(L, dtype=np.int32)
    for c, grp in enumerate(batch.groups):
        lab, nc = gen._components_after_outage(list(grp))
        sv, rb, _ = gen._resolve_references(lab, nc)
        labels[:, c], served[:, c], ref_bus[:, c], nis[c] = lab, sv, rb, nc
    return labels, served, ref_bus, nis


def main():
    ob.build_reference()
    fast = ob.load_reference("fastmath")
    strict = ob.load_reference("strict")
    assert fast is not None and strict is not None, "reference build unavailable"

    g = grid_118()
    S = timeseries_injections(g, 32)
    out = grid_arrays(g)
    out["S"] = S
    for tag, mod in (("fast", fast), ("strict", strict)):
        r = mod.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
        out[f"V_{tag}"], out[f"it_{tag}"], out[f"cv_{tag}"] = r["V"], r["iterations"], r["converged"]
    rng = np.random.default_rng(5)
    T = 48
    spread = np.linspace(0.0, 0.3, T)
    Vb = np.ascontiguousarray(g.V0[:, None] * np.exp(1j * spread[None, :] * rng.standard_normal((g.n, T))))
    Sb = np.ascontiguousarray(np.repeat(g.Sbus[:, None], T, axis=1))
    out["V0_bad"] = Vb
    for ls in (1, 0):
        for tag, mod in (("fast", fast), ("strict", strict)):
            r = mod.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(Sb, Vb, line_search=bool(ls))
            out[f"itbad{ls}_{tag}"], out[f"cvbad{ls}_{tag}"] = r["iterations"], r["converged"]
            if tag == "strict":
                out[f"Vbad{ls}_{tag}"] = r["V"]
    d = strict.debug_J(g.Yp, g.Yj, g.Yx, g.Sbus, g.V0, g.pv, g.pq)
    out.update(Jp=d["Jp"], Ji=d["Ji"], Jx=d["Jx"])
    np.savez_compressed(os.path.join(HERE, "golden_118.npz"), **out)

    g = grid_2000()
    S = timeseries_injections(g, 4)
    out = {k: v for k, v in grid_arrays(g).items() if k not in ("stamp", "stamp_pos", "f", "t")}
    out["S"] = S
    for tag, mod in (("fast", fast), ("strict", strict)):
        r = mod.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
        out[f"V_{tag}"], out[f"it_{tag}"], out[f"cv_{tag}"] = r["V"], r["iterations"], r["converged"]
    np.savez_compressed(os.path.join(HERE, "golden_2000.npz"), **out)

    g = grid_118()
    batch = contingency.build_batch(g)
    prio = np.zeros(g.n)
    prio[g.pv] = g.p_gen[g.pv]
    labels, served, ref_bus, nis = reference_islands(g, batch, prio)
    lo, so, ro, no = oi.islands(g.n, g.f, g.t, batch.live, batch.groups, g.ref, True, prio)
    assert np.array_equal(lo, labels) and np.array_equal(so, served) and np.array_equal(ro, ref_bus)
    assert np.array_equal(no, nis)
    V0, pin = contingency.start_and_pins(batch, g.V0, served, ref_bus)
    Yx = batch.Yx_matrix
    out = grid_arrays(g)
    out.update(labels=labels, served=served, ref_bus=ref_bus, n_islands=nis, V0n1=V0, pin=pin)
    for tag, mod in (("fast", fast), ("strict", strict)):
        r = mod.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch_contingency(
            np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx)), g.Sbus, V0, pin)
        out[f"V_{tag}"], out[f"it_{tag}"], out[f"cv_{tag}"] = r["V"], r["iterations"], r["converged"]
    np.savez_compressed(os.path.join(HERE, "golden_n1_118.npz"), **out)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
