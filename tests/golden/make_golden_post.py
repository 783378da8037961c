"""Generate golden_post.npz from the REFERENCE's own element models and post-processing.

Runs, from the reference checkout (imported through refstubs: numba, pandas and pandapower
replaced by minimal stand-ins, the reference's source unchanged):

* ``TransmissionLineModel`` / ``TwoWindingTransformerModel`` (p3s/models/, "t" transformer model,
  tap-characteristic lookup, rated-voltage ratios, phase shifters), ``TwoPort._apply_in_service``
  and ``apply_open_ends`` (Kron elimination of open ends), ``create_y_matrix`` /
  ``create_y_dc_matrix`` summed as ``NewtonPowerflowCpp.make_ybus`` does (p3s/NewtonPowerflowCpp.py:
  64-161) -> the Ybus, the DC susceptance matrix Bbus and the phase-shift injection;
* ``dc_initial_voltage`` (p3s/timeseries.py:200-247) with ``NewtonPowerflowCpp._pre_dc_solve``
  (:422-440) on that Bbus, for the base injections and four scenarios;
* ``compute_branch_loading`` (p3s/contingency/find_overloads.py:128-260) for the line and the
  transformer table over the first 64 cases of the 118-bus N-1 voltages of golden_n1_118.npz
  (two of them marked not converged).

Inputs: element tables on the seeded 118-bus grid's branches (12 of them transformers; some
out of service, some with an open end), bus shunts, and the grid's injections and start.

Usage (needs the reference checkout and pybind11): python tests/golden/make_golden_post.py
"""

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "parallel-pandapower-solver_gb300"), ROOT, HERE]

import refstubs  # noqa: E402
from p3s_gb300.synthetic import grid_118  # noqa: E402


class Column(np.ndarray):
    @property
    def values(self):
        return np.asarray(self)

    def to_numpy(self, dtype=None, copy=False):
        return np.array(self, dtype=dtype) if dtype is not None else np.asarray(self)

    def fillna(self, v):
        a = np.asarray(self)
        if a.dtype.kind == "f":
            a = np.where(np.isnan(a), v, a)
        return a.view(Column)


class _Index:
    def __init__(self, rows):
        self._rows = list(rows)

    def to_numpy(self):
        return np.asarray(self._rows)

    def get_indexer(self, keys):
        pos = {k: i for i, k in enumerate(self._rows)}
        return np.array([pos.get(tuple(k), -1) for k in keys])


class _Loc:
    def __init__(self, frame):
        self._f = frame

    def __getitem__(self, key):
        rows, col = key
        return np.asarray(self._f[col])[np.asarray(rows)].view(Column)


class Frame:
    """The columns of a table the reference's functions read, duck-typed."""

    def __init__(self, index=None, **cols):
        self._c = {k: np.asarray(v).view(Column) for k, v in cols.items()}
        n = len(next(iter(self._c.values())))
        self.index = _Index(range(n) if index is None else index)
        self.columns = list(self._c)
        self.loc = _Loc(self)

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
        return len(self.index.to_numpy())


class Net(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError:
            raise AttributeError(k) from None


def removable(g, rng, k):
    """k branches whose removal together keeps the grid connected (no DC island)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    keep = np.ones(g.n_branch, bool)
    out = []
    for b in rng.permutation(g.n_branch):
        keep[b] = False
        adj = coo_matrix((np.ones(keep.sum()), (g.f[keep], g.t[keep])), shape=(g.n, g.n))
        if connected_components(adj, directed=False)[0] == 1:
            out.append(int(b))
            if len(out) == k:
                break
        else:
            keep[b] = True
    return out


def inputs(seed=21):
    g = grid_118()
    rng = np.random.default_rng(seed)
    m = g.n_branch
    cut = removable(g, rng, 18)  # branches out of service or with an open end
    tr = np.sort(np.r_[cut[:3], rng.choice(np.setdiff1d(np.arange(m), cut), 9, replace=False)])
    ln = np.setdiff1d(np.arange(m), tr)
    nl, nt = len(ln), len(tr)
    lcut = [int(np.searchsorted(ln, b)) for b in cut[3:] if b in set(ln.tolist())]
    tcut = [int(np.searchsorted(tr, b)) for b in cut[:3]]
    bus_vn = np.full(g.n, 110.0)
    line = dict(from_bus=g.f[ln], to_bus=g.t[ln], length_km=rng.uniform(2.0, 40.0, nl),
                r_ohm_per_km=rng.uniform(0.03, 0.12, nl), x_ohm_per_km=rng.uniform(0.3, 0.42, nl),
                c_nf_per_km=rng.uniform(8.0, 12.0, nl), g_us_per_km=np.where(rng.random(nl) < 0.1, 0.5, 0.0),
                parallel=rng.choice([1, 1, 1, 2], nl), in_service=~np.isin(np.arange(nl), lcut[:5]),
                max_i_ka=rng.uniform(0.4, 1.2, nl), outage_group=[f"c{b + 1}" for b in ln])
    vk = rng.uniform(8.0, 14.0, nt)
    vk[3] = -10.0  # a negative short-circuit reactance (equivalent transformers)
    pfe = rng.uniform(20.0, 80.0, nt)
    i0 = rng.uniform(0.03, 0.08, nt)
    pfe[5], i0[5] = 0.0, 0.0  # no magnetising branch
    side = np.array(["hv", "lv", None, "hv", "lv", "hv", "hv", None, "lv", "hv", "lv", "hv"], dtype=object)
    trafo = dict(hv_bus=g.f[tr], lv_bus=g.t[tr], vn_hv_kv=110.0 * rng.uniform(0.98, 1.05, nt),
                 vn_lv_kv=110.0 * rng.uniform(0.98, 1.02, nt), sn_mva=rng.uniform(40.0, 250.0, nt), vk_percent=vk,
                 vkr_percent=rng.uniform(0.2, 0.5, nt), pfe_kw=pfe, i0_percent=i0,
                 shift_degree=np.where(np.arange(nt) == 2, 30.0, np.where(np.arange(nt) == 7, -150.0, 0.0)),
                 tap_pos=rng.integers(-3, 4, nt).astype(float), id_characteristic_table=rng.integers(0, 2, nt),
                 tap_side=list(side), in_service=np.arange(nt) != tcut[0], outage_group=[f"c{b + 1}" for b in tr])
    keys = [(cid, step) for cid in (0, 1) for step in range(-5, 6)]
    tap = dict(vk_percent=[10.0 + 0.1 * s for _, s in keys], vkr_percent=[0.35 + 0.01 * s for _, s in keys],
               angle_deg=[(2.0 * s if c == 1 else 0.0) for c, s in keys],
               voltage_ratio=[1.0 + 0.0125 * s for _, s in keys])
    open_line = np.zeros((nl, 2), bool)
    open_line[lcut[5:8], 0] = True
    open_line[lcut[8:11], 1] = True
    open_line[lcut[11], :] = True  # both ends open
    open_trafo = np.zeros((nt, 2), bool)
    open_trafo[tcut[1], 1] = True
    open_trafo[tcut[2], 0] = True
    shunt = np.zeros(g.n, complex)
    shunt[g.pq[:6]] = 1j * rng.uniform(0.01, 0.05, 6)
    return g, tr, ln, bus_vn, line, trafo, keys, tap, open_line, open_trafo, shunt


def on_pattern(g, M):
    """Values of a CSR matrix at the grid's Ybus positions (asserting nothing lies outside)."""
    M = M.tocsr()
    M.sum_duplicates()
    rows = np.repeat(np.arange(g.n), np.diff(g.Yp))
    vals = np.asarray(M[rows, g.Yj]).ravel()
    assert abs(M).sum() - np.abs(vals).sum() < 1e-9 * max(abs(M).sum(), 1.0)
    return vals


def main():
    refstubs.install()
    from scipy.sparse import coo_matrix

    from p3s import timeseries
    from p3s.contingency.find_overloads import compute_branch_loading
    from p3s.models.TransmissionLineModel import TransmissionLineModel
    from p3s.models.TwoWindingTransformerModel import TwoWindingTransformerModel
    from p3s.NewtonPowerflowCpp import NewtonPowerflow as NewtonPowerflowCpp

    g, tr, ln, bus_vn, line, trafo, keys, tap, open_line, open_trafo, shunt = inputs()
    sn_mva, f_hz = 100.0, 50.0
    bus = Frame(vn_kv=bus_vn)
    lt = Frame(**line)
    tt = Frame(**trafo)
    tapt = Frame(index=keys, **tap)
    lines = TransmissionLineModel(lt, bus_vn[line["from_bus"]], f_hz=f_hz, sn_mva=sn_mva)
    lines.apply_open_ends(open_line)
    trafos = TwoWindingTransformerModel(tt, bus, tapt, trafo_model="t", sn_mva=sn_mva)
    trafos.apply_open_ends(open_trafo)
    parts = [lines.create_y_matrix(n_bus=g.n), trafos.create_y_matrix(n_bus=g.n)]
    dat = np.concatenate([p.data for p in parts] + [shunt[shunt != 0]])
    row = np.concatenate([p.row for p in parts] + [np.nonzero(shunt)[0]])
    col = np.concatenate([p.col for p in parts] + [np.nonzero(shunt)[0]])
    Ybus = coo_matrix((dat, (row, col)), shape=(g.n, g.n)).tocsr()
    dparts = [lines.create_y_dc_matrix(n_bus=g.n), trafos.create_y_dc_matrix(n_bus=g.n)]
    Bbus = coo_matrix((np.concatenate([p.data for p in dparts]),
                       (np.concatenate([p.row for p in dparts]), np.concatenate([p.col for p in dparts]))),
                      shape=(g.n, g.n)).tocsr().imag
    p_shift = np.asarray(trafos.p_shift, dtype=float)

    # DC start of the base injections and four scenarios
    rng = np.random.default_rng(22)
    S_dc = np.repeat(g.Sbus[:, None], 5, axis=1)
    S_dc[g.pq, 1:] *= rng.uniform(0.7, 1.3, (len(g.pq), 4))
    V_dc = np.empty((g.n, 5), complex)
    for c in range(5):
        pf = types.SimpleNamespace(_initial_voltage=g.V0.copy(), busses={"ref": g.ref, "pv": g.pv, "pq": g.pq},
                                   _Bbus=Bbus, _sBus=S_dc[:, c].copy(), _p_shift=p_shift)
        pf._pre_dc_solve = types.MethodType(NewtonPowerflowCpp._pre_dc_solve, pf)
        V_dc[:, c] = timeseries.dc_initial_voltage(pf)

    # branch loading over the 118-bus N-1 voltages
    n1 = np.load(os.path.join(HERE, "golden_n1_118.npz"))
    V = np.where(n1["served"], n1["V_strict"], np.nan + 0j)[:, :64]  # the first 64 cases
    L = V.shape[1]
    conv = n1["cv_strict"].astype(bool)[:L].copy()
    conv[[7, 40]] = False
    res = types.SimpleNamespace(V=V, groups=[f"c{c}" for c in range(L)], converged=conv)
    net = Net(bus=bus, line=lt, trafo=tt, sn_mva=sn_mva)
    npf = types.SimpleNamespace(_ybus_elements={"line": lines, "trafo": trafos})
    out = {}
    for el in ("line", "trafo"):
        tab = compute_branch_loading(net, res, el, npf)
        for k in ("p_from_mw", "q_from_mvar", "p_to_mw", "q_to_mvar", "i_from_ka", "i_to_ka", "i_ka",
                  "loading_percent", "outaged"):
            out[f"{el}__res__{k}"] = np.asarray(getattr(tab, k))
    # text columns as fixed-width strings (no pickled objects): a missing tap side is ""
    for k, v in line.items():
        out[f"line__{k}"] = np.asarray(v)
    for k, v in trafo.items():
        out[f"trafo__{k}"] = np.asarray(["" if x is None else x for x in v]) if k == "tap_side" else np.asarray(v)
    for k, v in tap.items():
        out[f"tap__{k}"] = np.asarray(v)
    out.update(tap_keys=np.asarray(keys), trafo_branches=tr, line_branches=ln, bus_vn_kv=bus_vn,
               open_line=open_line, open_trafo=open_trafo, shunt=shunt, sn_mva=sn_mva, f_hz=f_hz,
               Ybus=on_pattern(g, Ybus), Bbus=on_pattern(g, Bbus.astype(complex)).real, p_shift=p_shift,
               S_dc=S_dc, V_dc=V_dc, V_flows=V, converged_flows=conv)
    np.savez_compressed(os.path.join(HERE, "golden_post.npz"), **out)
    print("golden_post.npz written:", {k: np.shape(v) for k, v in out.items() if np.ndim(v) > 1})


if __name__ == "__main__":
    main()
