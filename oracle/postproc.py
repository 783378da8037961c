"""Oracle for the steps either side of the Newton path (test infrastructure only).

* ``fill_sbus`` restates the reference's ``_fill_sbus`` (p3s/timeseries.py:122-141): every bus
  row starts at its base injection and takes its contributions in order, each
  ``coef * (x - base)`` added to the real or the imaginary part -- numpy, one contribution at
  a time over all time steps, the same IEEE operations as the reference's loop.
* ``branch_loading`` restates ``compute_branch_loading`` (p3s/contingency/find_overloads.py:
  128-260) with the branch admittance rows as scipy sparse matrices, like the reference.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def fill_sbus(s0, ptr, row, coef, base, imag, series):
    n = len(s0)
    T = series.shape[1]
    out = np.empty((n, T), dtype=np.complex128)
    re = np.repeat(np.asarray(s0).real[:, None], T, axis=1)
    im = np.repeat(np.asarray(s0).imag[:, None], T, axis=1)
    for i in range(n):
        for k in range(ptr[i], ptr[i + 1]):
            d = coef[k] * (series[row[k]] - base[k])
            if imag[k]:
                im[i] = im[i] + d
            else:
                re[i] = re[i] + d
    out.real = re
    out.imag = im
    return out


def branch_loading(n, f, t, y, V, converged, vn_from, vn_to, rating, kind, sn_mva, outaged):
    """(S_from, S_to, i_from, i_to, i_max, loading), each (nbr, L); outaged (nbr, L) bool."""
    nbr = len(f)
    rows = np.repeat(np.arange(nbr), 2)
    yf = sp.csr_matrix((np.c_[y[:, 0], y[:, 1]].ravel(), (rows, np.c_[f, t].ravel())), shape=(nbr, n))
    yt = sp.csr_matrix((np.c_[y[:, 2], y[:, 3]].ravel(), (rows, np.c_[f, t].ravel())), shape=(nbr, n))
    yf.sort_indices()
    yt.sort_indices()
    S_from = np.conj(yf @ V) * V[f, :] * sn_mva
    S_to = np.conj(yt @ V) * V[t, :] * sn_mva
    vm = np.abs(V)
    sqrt3 = np.sqrt(3.0)
    vf = np.asarray(vn_from, dtype=float)[:, None]
    vt = np.asarray(vn_to, dtype=float)[:, None]
    with np.errstate(divide="ignore", invalid="ignore"):
        i_from = np.abs(S_from) / (vf * vm[f, :] * sqrt3)
        i_to = np.abs(S_to) / (vt * vm[t, :] * sqrt3)
        i_max = np.maximum(i_from, i_to)
        line = np.asarray(kind)[:, None] == 0
        s_max = np.maximum(i_from * vf * sqrt3, i_to * vt * sqrt3)
        loading = np.where(line, i_max / np.asarray(rating, float)[:, None] * 100.0,
                           s_max / np.asarray(rating, float)[:, None] * 100.0)
    for arr in (S_from, S_to, i_from, i_to, i_max, loading):
        arr[outaged] = 0.0
    bad = ~np.asarray(converged, dtype=bool)
    for arr in (S_from, S_to, i_from, i_to, i_max, loading):
        arr[:, bad] = np.nan
    return S_from, S_to, i_from, i_to, i_max, loading


def dc_initial_voltage(Yp, Yj, Yx, pv, pq, ref, Pinj, V0):
    """``dc_initial_voltage`` / ``_pre_dc_solve`` (p3s/timeseries.py:200-247,
    NewtonPowerflowCpp.py:422-440): B[pvpq, pvpq] theta = Pinj[pvpq] - B[pvpq, ref] theta_ref
    with B the branch susceptance Laplacian (-Im Ybus off the diagonal, the diagonal their
    negated row sum), scipy spsolve; magnitudes kept from V0."""
    import scipy.sparse.linalg as spl

    n = len(Yp) - 1
    Y = sp.csr_matrix((np.asarray(Yx), Yj, Yp), shape=(n, n)).tocoo()
    off = Y.row != Y.col
    B = sp.coo_matrix((-Y.data.imag[off], (Y.row[off], Y.col[off])), shape=(n, n)).tocsr()
    B = (B - sp.diags(np.asarray(B.sum(axis=1)).ravel())).tocsr()
    pvpq = np.r_[pv, pq]
    theta_ref = np.angle(V0[ref])
    rhs = Pinj[pvpq] - B[pvpq, :][:, ref] @ theta_ref
    th = np.real(spl.spsolve(B[pvpq, :][:, pvpq].tocsc(), rhs))
    V = np.asarray(V0, dtype=np.complex128).copy()
    V[pvpq] = np.abs(V0[pvpq]) * np.exp(1j * th)
    return V


def branch_stamps(ys, y_from, y_to, a, b, in_service, open_from, open_to):
    """The general two-port's stamps (p3s/models/TwoWindingTransformerModel.py:172-175), the
    out-of-service mask (TwoPort.py:51-66) and the open-end Kron elimination
    (TwoPort.py:69-105), in numpy."""
    ff = (ys + y_from) / np.abs(a) ** 2
    ft = -ys / (np.conj(a) * np.conj(b))
    tf = -ys / (a * b)
    tt = (ys + y_to) / np.abs(b) ** 2
    ins = np.asarray(in_service, dtype=bool)
    ff, ft, tf, tt = (np.where(ins, v, 0.0) for v in (ff, ft, tf, tt))
    of, ot = np.asarray(open_from, dtype=bool), np.asarray(open_to, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore"):
        ff_red = np.where(tt != 0, ff - ft * tf / tt, ff)
        tt_red = np.where(ff != 0, tt - tf * ft / ff, tt)
    ff_new = np.where(of, 0.0, np.where(ot, ff_red, ff))
    tt_new = np.where(ot, 0.0, np.where(of, tt_red, tt))
    either = of | ot
    return np.stack([ff_new, np.where(either, 0.0, ft), np.where(either, 0.0, tf), tt_new], axis=1)


def ybus_from_stamps(n, f, t, stamps, bus_shunt):
    """COO sum of the stamps and shunts (TwoPort.py:133-149 create_y_matrix) as CSR."""
    rows = np.concatenate([f, f, t, t, np.arange(n)])
    cols = np.concatenate([f, t, f, t, np.arange(n)])
    data = np.concatenate([stamps[:, 0], stamps[:, 1], stamps[:, 2], stamps[:, 3], bus_shunt])
    Y = sp.coo_matrix((data, (rows, cols)), shape=(n, n)).tocsr()
    Y.sum_duplicates()
    Y.sort_indices()
    return Y
