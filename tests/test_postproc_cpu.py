"""The steps either side of the path, host side: the contribution list of the time-series
injection matrix (restated from the reference's build_sbus_matrix) and the oracle's
_fill_sbus reproduce the reference's own output bit for bit (golden_sbus.npz, made by
tests/golden/make_golden_sbus.py from the reference's p3s/timeseries.py)."""

import os

import numpy as np

from oracle.postproc import fill_sbus
from p3s_gb300.timeseries import contributions

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_sbus.npz")


def golden_inputs():
    d = np.load(GOLDEN)
    elements = {}
    for k in d.files:
        if "__" in k and not k.startswith("ts__"):
            name, col = k.split("__")
            elements.setdefault(name, {})[col] = d[k]
    ts = {(k.split("__")[1], k.split("__")[2]): d[k] for k in d.files if k.startswith("ts__")}
    return d, elements, ts


def test_oracle_sbus_matches_the_reference_bit_for_bit():
    d, elements, ts = golden_inputs()
    T, ptr, row, coef, base, imag, series = contributions(len(d["s0"]), elements, ts, float(d["sn_mva"]))
    assert T == d["Sbus"].shape[1] == 48  # the shortest series sets T
    assert ptr[-1] == len(row) and (np.diff(ptr) >= 0).all()
    S = fill_sbus(d["s0"], ptr, row, coef, base, imag, series)
    assert np.array_equal(S, d["Sbus"])
    # an out-of-service load injects nothing whatever its series says
    load = elements["load"]
    off = np.nonzero(~load["in_service"].astype(bool) & (load["bus"] >= 0))[0]
    assert len(off) > 0


POST = os.path.join(os.path.dirname(__file__), "golden", "golden_post.npz")


def golden_two_ports():
    """Two-port parameters of the golden element tables (lines and transformers in branch
    order) from the package's element-table helpers, with the flags the stamps take."""
    from p3s_gb300 import ybus

    d = np.load(POST)
    ln, tr = d["line_branches"], d["trafo_branches"]
    m = len(ln) + len(tr)
    vn = d["bus_vn_kv"]
    sn, fz = float(d["sn_mva"]), float(d["f_hz"])
    L = ybus.line_two_port(d["line__r_ohm_per_km"], d["line__x_ohm_per_km"], d["line__c_nf_per_km"],
                           d["line__g_us_per_km"], d["line__length_km"], d["line__parallel"], vn[d["line__from_bus"]],
                           f_hz=fz, sn_mva=sn)
    key = {(int(c), int(p)): i for i, (c, p) in enumerate(d["tap_keys"])}
    row = np.array([key[(int(c), int(p))] for c, p in zip(d["trafo__id_characteristic_table"], d["trafo__tap_pos"])])
    T = ybus.trafo_two_port(d["trafo__vn_hv_kv"], d["trafo__vn_lv_kv"], vn[d["trafo__hv_bus"]], vn[d["trafo__lv_bus"]],
                            d["trafo__sn_mva"], d["tap__vk_percent"][row], d["tap__vkr_percent"][row],
                            d["trafo__pfe_kw"], d["trafo__i0_percent"], d["trafo__shift_degree"],
                            d["tap__voltage_ratio"][row], d["tap__angle_deg"][row], tap_side=d["trafo__tap_side"],
                            sn_mva=sn)
    out = {}
    for k in ("ys", "y_from", "y_to", "a", "b", "ys_dc"):
        v = np.zeros(m, complex)
        v[ln], v[tr] = L[k], T[k]
        out[k] = v
    ins = np.ones(m, bool)
    ins[ln], ins[tr] = d["line__in_service"], d["trafo__in_service"]
    of, ot = np.zeros(m, bool), np.zeros(m, bool)
    of[ln], ot[ln] = d["open_line"][:, 0], d["open_line"][:, 1]
    of[tr], ot[tr] = d["open_trafo"][:, 0], d["open_trafo"][:, 1]
    out.update(in_service=ins, open_from=of, open_to=ot, p_shift_inj=T["p_shift_inj"])
    return d, out


def test_element_two_ports_rebuild_the_reference_ybus_and_bbus():
    """The package's element-table helpers (line / transformer two-ports, DC two-ports, phase
    shift) with the restated stamp formula and COO sum give the Ybus, Bbus and phase-shift
    injection the reference's own models built (golden_post.npz, make_golden_post.py), to 1e-13
    of the largest entry (the host divides complex numbers by another formula)."""
    from oracle.postproc import branch_stamps, ybus_from_stamps
    from p3s_gb300 import ybus
    from p3s_gb300.synthetic import grid_118

    d, tp = golden_two_ports()
    g = grid_118()
    flags = (tp["in_service"], tp["open_from"], tp["open_to"])
    st = branch_stamps(tp["ys"], tp["y_from"], tp["y_to"], tp["a"], tp["b"], *flags)
    Y = ybus_from_stamps(g.n, g.f, g.t, st, d["shunt"])
    rows = np.repeat(np.arange(g.n), np.diff(g.Yp))
    got = np.asarray(Y[rows, g.Yj]).ravel()
    assert np.abs(got - d["Ybus"]).max() <= 1e-13 * np.abs(d["Ybus"]).max()
    one = np.ones(len(tp["ys"]))
    dc = branch_stamps(tp["ys_dc"], 0 * one, 0 * one, one, one, *flags)
    B = ybus_from_stamps(g.n, g.f, g.t, dc, np.zeros(g.n)).imag
    gotB = np.asarray(B[rows, g.Yj]).ravel()
    assert np.abs(gotB - d["Bbus"]).max() <= 1e-13 * np.abs(d["Bbus"]).max()
    tr = d["trafo_branches"]
    ps = ybus.p_shift(g.n, g.f[tr], g.t[tr], tp["p_shift_inj"], d["trafo__in_service"], d["open_trafo"][:, 0],
                      d["open_trafo"][:, 1])
    assert np.abs(ps - d["p_shift"]).max() <= 1e-13 * np.abs(d["p_shift"]).max()
    assert (d["p_shift"] != 0).any() and (~tp["in_service"]).any() and tp["open_from"].any()
