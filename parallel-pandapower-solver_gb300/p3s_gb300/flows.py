"""Branch flows and loading of solved cases on the device
(p3s/contingency/find_overloads.py:128-260 ``compute_branch_loading``).

For every branch and case: the complex power at both ends from the branch's 2x2 admittance
and the solved voltages, the end currents |S| / (vn |V| sqrt 3), and the loading against the
line current rating (kA) or the transformer MVA rating -- the reference's formulas on array
grids. Outaged branches of a case report 0, non-converged cases NaN, NaN voltages (unserved
buses) propagate. One kernel over (branch, case); no per-case host work.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class BranchLoadingTable:
    groups: list
    p_from_mw: np.ndarray     # (n_branch, L)
    q_from_mvar: np.ndarray
    p_to_mw: np.ndarray
    q_to_mvar: np.ndarray
    i_from_ka: np.ndarray
    i_to_ka: np.ndarray
    i_ka: np.ndarray
    loading_percent: np.ndarray
    outaged: np.ndarray       # (n_branch, L) bool


def branch_flows(f, t, y, V, converged, vn_from, vn_to, rating, kind, sn_mva: float = 1.0, outages=None):
    """Raw flows: f, t (nbr,), y (nbr, 4) complex (Yff, Yft, Ytf, Ytt), V (n, L), converged (L,),
    vn_from / vn_to (kV) and rating (kA for kind 0 lines, MVA for kind 1 transformers) per
    branch, outages = (ptr (L+1,), idx) or None. Returns a dict of (nbr, L) arrays."""
    f = np.ascontiguousarray(f, dtype=np.int32)
    t = np.ascontiguousarray(t, dtype=np.int32)
    y = np.ascontiguousarray(y, dtype=np.complex128)
    V = np.ascontiguousarray(V, dtype=np.complex128)
    cv = np.ascontiguousarray(converged, dtype=np.uint8)
    n, L = V.shape
    nbr = len(f)
    vf = np.ascontiguousarray(np.broadcast_to(np.asarray(vn_from, dtype=np.float64), (nbr,)))
    vt = np.ascontiguousarray(np.broadcast_to(np.asarray(vn_to, dtype=np.float64), (nbr,)))
    rt = np.ascontiguousarray(np.broadcast_to(np.asarray(rating, dtype=np.float64), (nbr,)))
    kd = np.ascontiguousarray(np.broadcast_to(np.asarray(kind, dtype=np.uint8), (nbr,)))
    if y.shape != (nbr, 4) or t.shape != (nbr,) or cv.shape != (L,):
        raise ValueError("branch_flows: f, t (nbr,), y (nbr, 4), V (n, L), converged (L,)")
    op = oi = None
    if outages is not None:
        op = np.ascontiguousarray(outages[0], dtype=np.int32)
        oi = np.ascontiguousarray(outages[1], dtype=np.int32)
        if op.shape != (L + 1,):
            raise ValueError("branch_flows: outage pointers must be (L + 1,)")
    out = {k: np.empty((nbr, L), dtype=np.complex128) for k in ("S_from", "S_to")}
    out.update({k: np.empty((nbr, L)) for k in ("i_from", "i_to", "i_max", "loading")})
    rc = _lib.require_device().gbpf_branch_flows(
        n, nbr, L, _lib.i32(f), _lib.i32(t), _lib.cview(y), _lib.d(vf), _lib.d(vt), _lib.d(rt), _lib.u8(kd),
        float(sn_mva), _lib.cview(V), _lib.u8(cv), None if op is None else _lib.i32(op),
        None if oi is None else _lib.i32(oi), _lib.cview(out["S_from"]), _lib.cview(out["S_to"]),
        _lib.d(out["i_from"]), _lib.d(out["i_to"]), _lib.d(out["i_max"]), _lib.d(out["loading"]))
    _lib.check(rc, "branch_flows")
    return out


def compute_branch_loading(grid, res, vn_kv, rating, kind=0, sn_mva: float = 1.0, branches=None):
    """``compute_branch_loading`` for a ``ContingencyResultTable`` of an array grid: rows are
    ``branches`` (default: all of the grid's branches), columns the result's cases; each case's
    outaged branches (its group) report 0. vn_kv: (n_branch,) nominal voltage or a
    (vn_from, vn_to) pair; rating: kA (kind 0, lines) or MVA (kind 1, transformers)."""
    from .contingency import outage_lists

    sel = np.arange(grid.n_branch) if branches is None else np.asarray(branches, dtype=np.int64)
    vn_from, vn_to = (vn_kv, vn_kv) if not isinstance(vn_kv, tuple) else vn_kv
    take = lambda a: np.asarray(a)[sel] if np.ndim(a) else a  # noqa: E731
    remap = -np.ones(grid.n_branch, dtype=np.int64)
    remap[sel] = np.arange(len(sel))
    ptr, idx = outage_lists(res.groups)
    L = len(res.groups)
    keep = remap[idx] >= 0
    case_of = np.repeat(np.arange(L), np.diff(ptr))
    optr = np.zeros(L + 1, dtype=np.int32)
    optr[1:] = np.cumsum(np.bincount(case_of[keep], minlength=L))
    oidx = remap[idx][keep].astype(np.int32)
    fl = branch_flows(grid.f[sel], grid.t[sel], grid.stamp[sel], res.V, res.converged, take(vn_from), take(vn_to),
                      take(rating), take(kind), sn_mva, (optr, oidx))
    outaged = np.zeros((len(sel), len(res.groups)), dtype=bool)
    for c in range(len(res.groups)):
        outaged[oidx[optr[c]:optr[c + 1]], c] = True
    return BranchLoadingTable(list(res.groups), fl["S_from"].real, fl["S_from"].imag, fl["S_to"].real,
                              fl["S_to"].imag, fl["i_from"], fl["i_to"], fl["i_max"], fl["loading"], outaged)
