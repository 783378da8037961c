"""Branch stamps on the device (p3s/models/TwoPort.py, TransmissionLineModel.py,
TwoWindingTransformerModel.py): the general two-port with complex ratios at both ends,
out-of-service masking and Kron elimination of open ends, computed per branch by the
``gbpf_branch_stamps`` kernel; ``GpuSolver.update_Y_from_branches`` sums them into the
resident Ybus. The element tables' unit conversions (ohm/km, nF/km, rated voltages) stay with
the caller, as in the reference's model constructors."""

from __future__ import annotations

import numpy as np

from . import _lib


def _c(a, m):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.complex128), (m,)))


def _u(a, m):
    return None if a is None else np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.uint8), (m,)))


def branch_stamps(ys, y_from=0.0, y_to=0.0, a=1.0, b=1.0, in_service=None, open_from=None, open_to=None):
    """(m, 4) complex stamps (Yff, Yft, Ytf, Ytt): ys series admittance (p.u.), y_from / y_to
    shunt admittance at each end, a / b complex ratios at each end (tap * exp(j shift))."""
    ys = np.ascontiguousarray(np.asarray(ys, dtype=np.complex128).ravel())
    m = len(ys)
    arrs = [_c(x, m) for x in (ys, y_from, y_to, a, b)]
    flags = [_u(x, m) for x in (in_service, open_from, open_to)]
    out = np.empty((m, 4), dtype=np.complex128)
    rc = _lib.require_device().gbpf_branch_stamps(m, *[_lib.cview(x) for x in arrs],
                                                  *[None if f is None else _lib.u8(f) for f in flags], _lib.cview(out))
    _lib.check(rc, "branch_stamps")
    return out


# ------------------------------------------------------------------ element tables -> two-ports
def line_two_port(r_ohm_per_km, x_ohm_per_km, c_nf_per_km, g_us_per_km, length_km, parallel, vn_kv,
                  f_hz: float = 50.0, sn_mva: float = 1.0, model: str = "pi"):
    """Two-port parameters of lines from their table columns (p3s/models/TransmissionLineModel.py:
    14-51 pi_model, 54-98 t_model, 101-150 the model's constructor): ``ys`` series admittance,
    ``y_from`` = ``y_to`` shunt admittance at each end (p.u. of sn_mva), ``a`` = ``b`` = 1, and
    ``ys_dc``: the two-port whose stamps are the line's DC stamps (-1/x on the diagonal, +1/x off
    it, x the series reactance in p.u.). A T-model line is returned as its equivalent pi."""
    R, X = np.asarray(r_ohm_per_km, float), np.asarray(x_ohm_per_km, float)
    Cn, G = np.asarray(c_nf_per_km, float), np.asarray(g_us_per_km, float)
    length, par, vn = np.asarray(length_km, float), np.asarray(parallel, float), np.asarray(vn_kv, float)
    Z_N = (vn ** 2) / sn_mva
    B = 2 * Cn * f_hz * np.pi * 1e-9 * Z_N
    x_s = 1j * X * length / Z_N
    ys = 1 / (R * length / Z_N + x_s) / par  # series admittance
    ysh = 0.5 * (G * 1e-6 + 1j * B) * length * par  # half the shunt admittance
    if model == "t":
        a1 = a2 = 1.0 / (ys / 2)
        D = 2 * ysh + a1 + a2
        yft = -(a1 * a2) / D
        ys, ysh = -yft, (a1 - a1 * a1 / D) + yft
    elif model != "pi":
        raise ValueError(f"line model {model!r}: 'pi' or 't'")
    return {"ys": ys, "y_from": ysh, "y_to": ysh, "a": np.ones_like(ys), "b": np.ones_like(ys), "ys_dc": -(1 / x_s)}


def trafo_two_port(vn_hv_kv, vn_lv_kv, vn_bus_hv_kv, vn_bus_lv_kv, sn_trafo_mva, vk_percent, vkr_percent, pfe_kw,
                   i0_percent, shift_degree, tap_ratio, tap_angle_deg, tap_side=None, tap_side2=None,
                   sn_mva: float = 1.0, model: str = "t"):
    """Two-port parameters of two-winding transformers (p3s/models/TwoWindingTransformerModel.py:
    12-228): the rated-voltage ratio n0 and impedance base k, the short-circuit impedance (sign of
    vk kept), the magnetising admittance, the tap N = ratio exp(j (angle + shift)) on the side that
    carries it (hv: a, lv: b; no side: the shift on a), and for the "t" model pandapower's
    wye-delta conversion to a pi. The tap-table columns (vk, vkr, angle, ratio) are the ones of
    each transformer's (characteristic, tap position) row, looked up by the caller. Returns
    ``ys``, ``y_from``, ``y_to``, ``a``, ``b`` (the stamps of the general two-port), ``ys_dc`` (the
    two-port of its DC stamps, 1 / (x tap)) and ``p_shift_inj`` (the DC phase-shift injection,
    + at hv / - at lv)."""
    f = lambda v: np.asarray(v, dtype=float)  # noqa: E731
    vn_ratio_hv = f(vn_hv_kv) / f(vn_bus_hv_kv)
    vn_ratio_lv = f(vn_lv_kv) / f(vn_bus_lv_kv)
    n0 = vn_ratio_hv / vn_ratio_lv
    k = vn_ratio_lv ** 2
    angle_deg = f(tap_angle_deg)
    side = None if tap_side is None else np.asarray(tap_side, dtype=object)
    if side is not None:
        angle_deg = np.where(side == "lv", -angle_deg, angle_deg)
    theta = np.deg2rad(angle_deg + f(shift_degree))
    N = f(tap_ratio) * np.exp(1j * theta)
    a = np.ones_like(N)
    b = np.ones_like(N)
    if side is not None:
        a = np.where(side == "hv", N, 1.0)
        b = np.where(side == "lv", N, 1.0)
        a = np.where(~np.isin(side, ("hv", "lv")), N, a)
    if tap_side2 is not None:
        side2 = np.asarray(tap_side2, dtype=object)
        a = np.where(side2 == "hv", N, a)
        b = np.where(side2 == "lv", N, b)
    a = a * n0
    sn_scaled = sn_mva / f(sn_trafo_mva)
    z_sc = f(vk_percent) / 100.0 * sn_scaled * k
    r_sc = f(vkr_percent) / 100.0 * sn_scaled * k
    x_sc = np.sign(z_sc) * np.sqrt(z_sc ** 2 - r_sc ** 2)
    z_k = r_sc + 1j * x_sc
    i_0 = f(i0_percent) / 100.0 * f(sn_trafo_mva)
    pfe_mw = f(pfe_kw) / 1000.0
    g_m = pfe_mw / sn_mva
    b_m_squared = np.square(i_0) - np.square(pfe_mw)
    with np.errstate(invalid="ignore"):
        b_m = np.where(b_m_squared < 0, 0, np.sqrt(b_m_squared) / sn_mva)
    y_ = (g_m - 1j * b_m) / k
    if model == "pi":  # no tap in the reference's pi stamp
        z_ = 1 / z_k
        ys, y_from, y_to = z_, y_ / 2.0, y_ / 2.0
        a_st, b_st = np.ones_like(N), np.ones_like(N)
    elif model == "t":
        has_mag = y_ != 0
        za = zb = z_k / 2.0
        zc = 1.0 / np.where(has_mag, y_, 1.0)
        zsum = za * zb + za * zc + zb * zc
        ys = 1.0 / np.where(has_mag, zsum / zc, z_k)
        y_from = np.where(has_mag, zb / zsum, 0.0)
        y_to = np.where(has_mag, za / zsum, 0.0)
        a_st, b_st = a, b
    else:
        raise ValueError(f"transformer model {model!r}: 't' or 'pi'")
    one_over_x = 1 / (1j * x_sc)
    b_dc = one_over_x / (np.abs(a) * np.abs(b))
    p_shift_inj = theta / (x_sc * np.abs(a) * np.abs(b))
    return {"ys": ys, "y_from": y_from, "y_to": y_to, "a": a_st, "b": b_st, "ys_dc": -b_dc,
            "p_shift_inj": p_shift_inj}


def p_shift(n, f, t, p_shift_inj, in_service=None, open_from=None, open_to=None):
    """Per-bus DC phase-shift injection (TwoWindingTransformerModel.py:206-228, TwoPort.py:107-112):
    + at the from bus and - at the to bus of every transformer in service with both ends closed."""
    inj = np.asarray(p_shift_inj, dtype=float).copy()
    if in_service is not None:
        inj = np.where(np.asarray(in_service, bool), inj, 0.0)
    if open_from is not None or open_to is not None:
        m = len(inj)
        of = np.zeros(m, bool) if open_from is None else np.asarray(open_from, bool)
        ot = np.zeros(m, bool) if open_to is None else np.asarray(open_to, bool)
        inj = np.where(of | ot, 0.0, inj)
    out = np.zeros(n)
    np.add.at(out, np.asarray(f, dtype=np.intp), inj)
    np.add.at(out, np.asarray(t, dtype=np.intp), -inj)
    return out
