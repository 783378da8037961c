"""Generate golden_floor.json: how far the REFERENCE's own two builds of nr_klu differ on the
large grids of the full-size parity tests.

The reference's p3s/cpp/nr_klu.cpp is compiled twice by oracle/build.py -- with its release
flags (-O3 -funroll-loops -ffast-math, p3s/cpp/CMakeLists.txt:32-35) and with strict IEEE
arithmetic (-ffp-contract=off) -- against the same KLU-API shim, so both use the same pivot
order and differ only by floating-point contraction and reassociation. On grids of 15,000
buses and more that alone moves the solved voltages by 1e-11 .. 1e-10 p.u. (identical
iterations): a double-precision answer of another code is held to a multiple of this floor
there instead of to 1e-11, which the reference does not reproduce itself.

Per grid (keyed by its bus count): the largest |V_release - V_strict| over 16 load scenarios
(base loads x U(0.8, 1.2), solved from the grid's flat start, tol 1e-8); and for the 2,000-bus
grid near its loading limit ("2000x7.5": 16 cases loaded 7.5x; "n1_2000x6": the N-1 sweep
loaded 6x) over the cases both builds converge.

Usage (needs the reference checkout and pybind11): python tests/golden/make_golden_floor.py
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "parallel-pandapower-solver_gb300"), ROOT, os.path.dirname(HERE)]

from oracle import build as ob  # noqa: E402


def large_grids():
    from p3s_gb300.synthetic import make_grid, scenario_injections
    from test_gpu_full_size import _large_multigrid_grids, _serving_sizes

    out = [g for g, _ in _large_multigrid_grids()]
    sizes = _serving_sizes()
    out += [make_grid(int(sizes[i]), seed=500 + i, max_drop_pu=0.05) for i in range(len(sizes) - 3, len(sizes))]
    return [(g, scenario_injections(g, 16, seed=11)) for g in out]


def stressed_cases():
    """The 2,000-bus grid near its loading limit: 16 cases loaded 7.5x (x 0.95 .. 1.05) and the
    full N-1 sweep loaded 6x (flat start, islands re-slacked), keyed as the tests key them."""
    from oracle import islands as oisl
    from p3s_gb300 import contingency
    from p3s_gb300.synthetic import grid_2000

    g = grid_2000()
    S = np.ascontiguousarray(np.repeat(g.Sbus[:, None] * 7.5, 16, axis=1) * np.linspace(0.95, 1.05, 16)[None, :])
    batch = contingency.build_batch(g)
    prio = np.zeros(g.n)
    prio[g.pv] = np.maximum(g.p_gen[g.pv], np.finfo(float).tiny)
    _, served, rb, _ = oisl.islands(g.n, g.f, g.t, batch.live, batch.groups, g.ref, True, prio)
    V0, pin = oisl.start_and_pins(g.V0, served, rb, g.ref)
    Yx = batch.Yx_matrix
    return g, S, (np.ascontiguousarray(np.abs(Yx)), np.ascontiguousarray(np.angle(Yx)), g.Sbus * 6.0, V0, pin, served)


def main():
    ob.build_reference()
    fast, strict = ob.load_reference("fastmath"), ob.load_reference("strict")
    floor = {}
    g, S, (mag, ang, S6, V0, pin, served) = stressed_cases()
    f = fast.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
    s = strict.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
    ok = f["converged"] & s["converged"]
    assert np.array_equal(f["converged"], s["converged"]) and ok.any()
    floor["2000x7.5"] = float(np.abs(f["V"][:, ok] - s["V"][:, ok]).max())
    f = fast.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch_contingency(mag, ang, S6, V0, pin)
    s = strict.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch_contingency(mag, ang, S6, V0, pin)
    ok = f["converged"] & s["converged"]
    assert np.array_equal(f["converged"], s["converged"])
    d = np.where(served[:, ok], np.abs(f["V"][:, ok] - s["V"][:, ok]), 0.0)
    floor["n1_2000x6"] = float(d.max())
    print(floor)
    for g, S in large_grids():
        f = fast.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
        s = strict.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(S, g.V0)
        assert f["converged"].all() and s["converged"].all()
        assert np.array_equal(f["iterations"], s["iterations"])
        floor[str(g.n)] = float(np.abs(f["V"] - s["V"]).max())
        print(g.n, floor[str(g.n)])
    with open(os.path.join(HERE, "golden_floor.json"), "w") as fh:
        json.dump(floor, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
