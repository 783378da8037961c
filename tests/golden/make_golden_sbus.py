"""Generate golden_sbus.npz from the REFERENCE's own build_sbus_matrix / _fill_sbus.

Imports p3s/timeseries.py from the reference checkout with numba replaced by a stand-in whose
``njit`` returns the function unchanged and ``prange`` is ``range`` (the kernel then runs as
plain Python, the same arithmetic), and calls ``build_sbus_matrix(pf, net, timeseries)`` with a
duck-typed solver (``_sBus``) and a duck-typed net whose element tables carry exactly the
columns the function reads (``_lookup``, ``p_mw``, ``q_mvar``, ``scaling``, ``in_service``).
Inputs: the seeded 118-bus grid with loads (two per PQ bus on a few buses, some out of
service, one unsupplied), static generators and generators, 48 hourly steps.

Usage (needs the reference checkout): python tests/golden/make_golden_sbus.py
"""

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "parallel-pandapower-solver_gb300"), ROOT]

from oracle import build as ob  # noqa: E402
from p3s_gb300.synthetic import grid_118  # noqa: E402


class Column(np.ndarray):
    def to_numpy(self, dtype=None):
        return np.asarray(self, dtype=dtype)


class Frame:
    def __init__(self, **cols):
        self._c = {k: np.asarray(v).view(Column) for k, v in cols.items()}

    def __getitem__(self, k):
        return self._c[k]

    def __getattr__(self, k):
        try:
            return self.__dict__["_c"][k]
        except KeyError:
            raise AttributeError(k) from None

    def __contains__(self, k):
        return k in self._c

    def __len__(self):
        return len(next(iter(self._c.values())))


class Net(dict):
    sn_mva = 1.0


def reference_timeseries():
    nb = types.ModuleType("numba")
    nb.njit = lambda *a, **k: (a[0] if a and callable(a[0]) else (lambda f: f))
    nb.prange = range
    nb.set_num_threads = lambda n: None
    nb.get_num_threads = lambda: 1
    nb.config = types.SimpleNamespace(NUMBA_NUM_THREADS=1)
    typed = types.ModuleType("numba.typed")
    typed.List = list
    nb.typed = typed
    sys.modules["numba"] = nb
    sys.modules["numba.typed"] = typed
    path = os.path.join(ob.REF_CPP, "..", "timeseries.py")  # p3s/timeseries.py
    spec = importlib.util.spec_from_file_location("ref_timeseries", os.path.normpath(path))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def inputs(seed=3, T=48):
    g = grid_118()
    rng = np.random.default_rng(seed)
    pq, pv = g.pq, g.pv
    load_bus = np.r_[pq, pq[:10], -1]  # ten buses with a second load, one unsupplied load
    nl = len(load_bus)
    load = dict(bus=load_bus, p_mw=rng.uniform(0.1, 1.0, nl), q_mvar=rng.uniform(0.0, 0.4, nl),
                scaling=rng.choice([1.0, 0.8, 1.2], nl), in_service=rng.random(nl) > 0.05)
    sg_bus = pv[: len(pv) // 2]
    ns = len(sg_bus)
    sgen = dict(bus=sg_bus, p_mw=rng.uniform(0.1, 2.0, ns), q_mvar=np.zeros(ns), scaling=np.ones(ns),
                in_service=np.ones(ns, bool))
    gn = len(pv)
    gen = dict(bus=pv, p_mw=rng.uniform(0.2, 2.0, gn), scaling=rng.uniform(0.9, 1.1, gn), in_service=np.ones(gn, bool))
    ts = {
        ("load", "p_mw"): load["p_mw"][:, None] * rng.uniform(0.5, 1.5, (nl, T)),
        ("load", "q_mvar"): load["q_mvar"][:, None] * rng.uniform(0.5, 1.5, (nl, T)),
        ("sgen", "p_mw"): sgen["p_mw"][:, None] * rng.uniform(0.0, 1.2, (ns, T)),
        ("gen", "p_mw"): gen["p_mw"][:, None] * rng.uniform(0.6, 1.1, (gn, T + 5)),  # longer: T = min
    }
    return g, dict(load=load, sgen=sgen, gen=gen), ts


def main():
    mod = reference_timeseries()
    g, elements, ts = inputs()
    net = Net()
    for name, tab in elements.items():
        cols = {("_lookup" if k == "bus" else k): v for k, v in tab.items()}
        net[name] = Frame(**cols)
    pf = types.SimpleNamespace(_sBus=g.Sbus)
    S = mod.build_sbus_matrix(pf, net, ts)
    out = {"s0": g.Sbus, "Sbus": S, "sn_mva": 1.0}
    for name, tab in elements.items():
        for k, v in tab.items():
            out[f"{name}__{k}"] = np.asarray(v)
    for (name, var), v in ts.items():
        out[f"ts__{name}__{var}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "golden_sbus.npz"), **out)
    print("golden_sbus.npz written", S.shape)


if __name__ == "__main__":
    main()
