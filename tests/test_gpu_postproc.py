"""Either side of the path on the GPU: the time-series injection matrix against the
reference's own output (bit for bit), and branch flows / loading of solved N-1 cases against
the restated compute_branch_loading (zeros and NaNs exactly; values to 1e-11 relative / 1e-10
absolute: a branch's end power is the small difference of terms ~|y| larger, so rounding of
the host's complex products -- which may fuse multiply-adds -- shows at ~1e-12)."""

import numpy as np
import pytest

from oracle.postproc import branch_loading
from p3s_gb300 import contingency
from p3s_gb300.flows import compute_branch_loading
from p3s_gb300.synthetic import grid_118
from p3s_gb300.timeseries import build_sbus_matrix
from test_postproc_cpu import golden_inputs

pytestmark = pytest.mark.gpu


def test_device_sbus_matches_the_reference_bit_for_bit():
    d, elements, ts = golden_inputs()
    S = build_sbus_matrix(d["s0"], elements, ts, float(d["sn_mva"]))
    assert np.array_equal(S, d["Sbus"])


def test_branch_loading_of_an_n1_sweep_matches_the_restated_reference():
    g = grid_118()
    res = contingency.solve_contingencies(g, reslack_islands=True)
    assert (~res.served).any() and res.converged.all()
    rng = np.random.default_rng(4)
    nbr = g.n_branch
    vn = rng.choice([110.0, 220.0], nbr)
    kind = (rng.random(nbr) < 0.2).astype(np.uint8)
    rating = np.where(kind == 0, rng.uniform(0.2, 1.0, nbr), rng.uniform(50, 300, nbr))
    conv = res.converged.copy()
    conv[5] = False  # a non-converged column is reported NaN
    res.converged = conv
    tab = compute_branch_loading(g, res, vn, rating, kind, sn_mva=100.0)
    outaged = np.zeros((nbr, len(res.groups)), bool)
    for c, grp in enumerate(res.groups):
        outaged[grp, c] = True
    assert np.array_equal(tab.outaged, outaged)
    ref = branch_loading(g.n, g.f, g.t, g.stamp, res.V, conv, vn, vn, rating, kind, 100.0, outaged)
    got = (tab.p_from_mw + 1j * tab.q_from_mvar, tab.p_to_mw + 1j * tab.q_to_mvar, tab.i_from_ka, tab.i_to_ka,
           tab.i_ka, tab.loading_percent)
    for a, b in zip(got, ref):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        assert np.array_equal(a[outaged & conv[None, :]], b[outaged & conv[None, :]])  # zeros
        m = ~np.isnan(b)
        assert np.allclose(a[m], b[m], rtol=1e-11, atol=1e-10)
    assert np.isnan(tab.loading_percent[:, 5]).all()
    # a branch touching an unserved bus has undefined flow
    c = int(np.nonzero((~res.served).any(axis=0))[0][0])
    dead = np.nonzero(~res.served[:, c])[0]
    touch = np.isin(g.f, dead) | np.isin(g.t, dead)
    touch &= ~outaged[:, c]
    assert np.isnan(tab.i_ka[touch, c]).all()


def test_dc_start_from_the_ybus_matches_the_restated_reference_and_starts_newton():
    from oracle import cpu
    from oracle.postproc import dc_initial_voltage
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.synthetic import grid_2000

    for g in (grid_118(), grid_2000()):
        s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
        V, used = s.dc_start(g.Sbus.real, g.V0)
        assert used
        ref = dc_initial_voltage(g.Yp, g.Yj, g.Yx, g.pv, g.pq, g.ref, g.Sbus.real, g.V0)
        assert np.abs(np.angle(V) - np.angle(ref)).max() < 1e-10
        assert np.array_equal(np.abs(V)[g.ref], np.abs(g.V0)[g.ref])
        r = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(g.Sbus[:, None], V)
        flat = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(g.Sbus[:, None], g.V0)
        assert r["converged"][0] and r["iterations"][0] <= flat["iterations"][0]


def test_ybus_from_branch_stamps_on_the_device():
    """Two-port stamps (taps, phase shifts, out of service, open ends) and their Ybus summed on
    the device against the restated reference models (1e-13 of the largest stamp: the Kron
    elimination of an open end subtracts nearly equal terms, and the host divides complex
    numbers by a different formula); a power flow on the device-built Ybus equals one on the
    same Ybus handed to update_Y (bit for bit)."""
    import scipy.sparse as sp

    from oracle.postproc import branch_stamps as ref_stamps
    from oracle.postproc import ybus_from_stamps
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.ybus import branch_stamps

    g = grid_118()
    m = g.n_branch
    rng = np.random.default_rng(8)
    x = 0.02 + 0.3 * rng.random(m)
    ys = 1.0 / (x * rng.uniform(0.1, 0.4, m) + 1j * x)
    ysh = 0.5j * rng.uniform(0.0, 0.05, m)
    tap = np.where(rng.random(m) < 0.1, rng.uniform(0.9, 1.1, m), 1.0)
    shift = np.where(rng.random(m) < 0.05, np.deg2rad(rng.uniform(-10, 10, m)), 0.0)
    a = tap * np.exp(1j * shift)
    ins = rng.random(m) > 0.03
    of = rng.random(m) < 0.03
    ot = rng.random(m) < 0.03
    st = branch_stamps(ys, ysh, ysh, a, 1.0, ins, of, ot)
    ref = ref_stamps(ys, ysh, ysh, a, np.ones(m), ins, of, ot)
    assert np.abs(st - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.array_equal(st == 0, ref == 0)
    shunt = np.zeros(g.n, complex)
    shunt[g.pq[:5]] = 0.02j
    Yref = ybus_from_stamps(g.n, g.f, g.t, ref, shunt)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    is_slack = np.zeros(g.n, np.uint8)
    is_slack[g.ref] = 1
    s.set_branches(g.f, g.t, g.stamp_pos, g.stamp, is_slack)
    s.update_Y_from_branches(st, shunt)
    # the device Ybus on the grid's pattern: entries outside Yref's pattern are zero
    Ydev = sp.csr_matrix((s.Yx, g.Yj, g.Yp), shape=(g.n, g.n))
    assert abs(Ydev - Yref).max() <= 1e-13 * abs(Yref).max()
    host = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    host.update_Y(s.Yx)
    p = GpuSolver.params()
    S = g.Sbus[:, None] * np.ones((1, 4))
    r1, r2 = s.solve_batch(S, g.V0, p), host.solve_batch(S, g.V0, p)
    assert np.array_equal(r1["V"], r2["V"]) and np.array_equal(r1["iterations"], r2["iterations"])


def _device_element_stamps():
    """Device stamps (AC and DC) of the golden element tables, and the solver holding the
    118-bus grid's branch table with the element Ybus summed on the device."""
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.ybus import branch_stamps
    from test_postproc_cpu import golden_two_ports

    d, tp = golden_two_ports()
    g = grid_118()
    flags = (tp["in_service"], tp["open_from"], tp["open_to"])
    st = branch_stamps(tp["ys"], tp["y_from"], tp["y_to"], tp["a"], tp["b"], *flags)
    dc = branch_stamps(tp["ys_dc"], 0.0, 0.0, 1.0, 1.0, *flags)
    s = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    is_slack = np.zeros(g.n, np.uint8)
    is_slack[g.ref] = 1
    s.set_branches(g.f, g.t, g.stamp_pos, g.stamp, is_slack)
    s.update_Y_from_branches(st, d["shunt"])
    return d, tp, g, st, dc, s


def test_ybus_from_element_tables_matches_the_reference_models():
    """Element tables -> two-ports (host) -> stamps with out-of-service masks and open-end Kron
    elimination -> Ybus summed, both on the device, against the Ybus the reference's own
    TransmissionLineModel / TwoWindingTransformerModel / create_y_matrix built (golden_post.npz);
    1e-13 of the largest entry (the device divides complex numbers by another formula)."""
    d, tp, g, st, dc, s = _device_element_stamps()
    assert np.abs(s.Yx - d["Ybus"]).max() <= 1e-13 * np.abs(d["Ybus"]).max()
    assert (st[~tp["in_service"]] == 0).all() and (st[tp["open_from"] | tp["open_to"]][:, 1:3] == 0).all()


def test_branch_loading_matches_the_reference_compute_branch_loading():
    """Branch flows of the reference's own compute_branch_loading (line and transformer tables,
    outaged branches 0, non-converged cases NaN, NaN voltages propagating) from the device
    stamps of the same element tables (values 1e-11 relative / 1e-10 absolute)."""
    from p3s_gb300.flows import branch_flows

    d, tp, g, st, dc, s = _device_element_stamps()
    V, conv = d["V_flows"], d["converged_flows"]
    L = V.shape[1]
    vn = d["bus_vn_kv"]
    for el, rows in (("line", d["line_branches"]), ("trafo", d["trafo_branches"])):
        local = -np.ones(g.n_branch, np.int64)
        local[rows] = np.arange(len(rows))
        # case c > 0 of the N-1 voltages has branch c - 1 out (its outage group)
        hit = [local[c - 1] if c > 0 and local[c - 1] >= 0 else -1 for c in range(L)]
        ptr = np.zeros(L + 1, np.int32)
        ptr[1:] = np.cumsum([h >= 0 for h in hit])
        idx = np.array([h for h in hit if h >= 0], np.int32)
        if el == "line":
            vf = vt = vn[d["line__from_bus"]]
            rating, kind = d["line__max_i_ka"], 0
        else:
            vf, vt = vn[d["trafo__hv_bus"]], vn[d["trafo__lv_bus"]]
            rating, kind = d["trafo__sn_mva"], 1
        got = branch_flows(g.f[rows], g.t[rows], st[rows], V, conv, vf, vt, rating, kind, float(d["sn_mva"]),
                           (ptr, idx))
        pairs = ((got["S_from"].real, "p_from_mw"), (got["S_from"].imag, "q_from_mvar"),
                 (got["S_to"].real, "p_to_mw"), (got["S_to"].imag, "q_to_mvar"), (got["i_from"], "i_from_ka"),
                 (got["i_to"], "i_to_ka"), (got["i_max"], "i_ka"), (got["loading"], "loading_percent"))
        out = d[f"{el}__res__outaged"]
        assert out.any()
        for a, k in pairs:
            b = d[f"{el}__res__{k}"]
            assert np.array_equal(np.isnan(a), np.isnan(b)), k
            assert np.array_equal(a[out & conv[None, :]], b[out & conv[None, :]]), k  # zeros
            m = ~np.isnan(b)
            assert np.allclose(a[m], b[m], rtol=1e-11, atol=1e-10), k


def test_batched_dc_start_matches_the_reference_dc_initial_voltage():
    """The reference's dc_initial_voltage (its own Bbus of DC branch stamps, phase-shift
    injection, _pre_dc_solve) for the base injections and four scenarios, against the device's
    batched DC start (B factored once from the device DC stamps, five substitutions): angles
    within 1e-10 rad, magnitudes kept; one column alone gives the same bits as in the batch."""
    d, tp, g, st, dc, s = _device_element_stamps()
    Pinj = np.ascontiguousarray(d["S_dc"].real + d["p_shift"][:, None])
    V, used = s.dc_start(Pinj, g.V0, dc_stamps=dc)
    assert used.all()
    ref = d["V_dc"]
    assert np.abs(np.angle(V * np.conj(ref))).max() < 1e-10
    assert np.allclose(np.abs(V), np.abs(ref), rtol=1e-15, atol=0)
    assert np.abs(np.angle(ref)).max() > 0.3  # phase shifters: the shift injection matters
    one, ok = s.dc_start(Pinj[:, 2], g.V0, dc_stamps=dc)
    assert ok and np.array_equal(one, V[:, 2])
    # the Ybus-derived B (the DC start without element data) still starts Newton
    V2, used2 = s.dc_start(np.ascontiguousarray(g.Sbus.real[:, None] * np.ones((1, 3))), g.V0)
    assert used2.all() and np.array_equal(V2[:, 0], V2[:, 2])
