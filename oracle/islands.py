"""Oracle for N-1 islanding and re-slacking (test infrastructure only).

Restates, with numpy/scipy, the reference's p3s/contingency/case_generator.py:
* ``_components_after_outage`` (:355-377): live branches minus the outage group, undirected
  adjacency, ``scipy.sparse.csgraph.connected_components`` labels;
* ``_resolve_references`` (:379-430): per component the lowest-index slack bus, else (with
  reslack) the generator chosen by the ranking -- here the highest priority (largest
  scheduled P), ties to the lowest bus index, in place of the reference's lowest
  short-circuit impedance -- else unserved;
* ``solver_cpp.py:119-134``: V0 / pin of re-slack references (|v0| + 0j) and unserved
  buses (1 + 0j).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components


def components_after_outage(n, f, t, live, outaged):
    keep = np.asarray(live, dtype=bool).copy()
    if len(outaged):
        keep[np.asarray(outaged, dtype=np.int64)] = False
    fk, tk = np.asarray(f)[keep], np.asarray(t)[keep]
    rows = np.concatenate([fk, tk])
    cols = np.concatenate([tk, fk])
    adj = sp.coo_matrix((np.ones(rows.shape[0], dtype=np.int8), (rows, cols)), shape=(n, n)).tocsr()
    n_comp, labels = connected_components(adj, directed=False)
    return labels.astype(np.int32), n_comp


def resolve_references(labels, n_comp, ref, reslack, prio):
    comp_ref = np.full(n_comp, -1, dtype=np.int64)
    ref = np.asarray(ref, dtype=np.int64)
    if len(ref):
        tmp = np.full(n_comp, np.iinfo(np.int64).max, dtype=np.int64)
        np.minimum.at(tmp, labels[ref], ref)
        has = tmp != np.iinfo(np.int64).max
        comp_ref[has] = tmp[has]
    if reslack:
        gens = np.nonzero(np.asarray(prio) > 0)[0]
        if len(gens):
            gc = labels[gens]
            best = np.full(n_comp, -np.inf)
            np.maximum.at(best, gc, prio[gens])
            need = (comp_ref == -1) & np.isfinite(best)
            is_best = (prio[gens] == best[gc]) & need[gc]
            cand = np.where(is_best, gens, np.iinfo(np.int64).max)
            chosen = np.full(n_comp, np.iinfo(np.int64).max, dtype=np.int64)
            np.minimum.at(chosen, gc, cand)
            picked = need & (chosen != np.iinfo(np.int64).max)
            comp_ref[picked] = chosen[picked]
    ref_bus = comp_ref[labels]
    return ref_bus != -1, ref_bus.astype(np.int32)


def islands(n, f, t, live, groups, ref, reslack, prio):
    """(labels, served, ref_bus, n_islands) for every case, as the device API returns them."""
    L = len(groups)
    labels = np.empty((n, L), dtype=np.int32)
    served = np.empty((n, L), dtype=bool)
    ref_bus = np.empty((n, L), dtype=np.int32)
    nis = np.empty(L, dtype=np.int32)
    for c, g in enumerate(groups):
        lab, nc = components_after_outage(n, f, t, live, g)
        s, r = resolve_references(lab, nc, ref, reslack, prio)
        labels[:, c], served[:, c], ref_bus[:, c], nis[c] = lab, s, r, nc
    return labels, served, ref_bus, nis


def start_and_pins(v_start, served, ref_bus, ref):
    """Per-case start voltages and pins of outage cases (n, L), for any start voltage.

    solver_cpp.py:119-134 pins a re-slack reference at |v0| + 0j and an unserved bus at
    1 + 0j, from a flat start where every other bus of a re-slacked island already has angle
    0. From a warm start (a converged base case) the whole re-slacked island is rotated by its
    new reference's angle, so that the reference sits at |v0| + 0j and the island's angle
    differences are kept; islands that hold a slack bus keep the start as it is. For a flat
    start this is exactly the reference's rule."""
    v_start = np.asarray(v_start, dtype=np.complex128)
    n, L = served.shape
    is_slack = np.zeros(n, dtype=bool)
    is_slack[np.asarray(ref, dtype=np.int64)] = True
    V0 = np.repeat(v_start[:, None], L, axis=1)
    pin = np.zeros((n, L), dtype=np.uint8)
    rb = np.asarray(ref_bus, dtype=np.int64)
    resl = served & ~is_slack[np.where(rb >= 0, rb, 0)]
    rot = np.exp(-1j * np.angle(v_start))  # e^{-j angle(v_r)} per candidate reference r
    V0[resl] = V0[resl] * rot[rb[resl]]
    bus = np.arange(n)[:, None]
    is_ref = resl & (rb == bus)
    V0[is_ref] = np.abs(np.broadcast_to(v_start[:, None], V0.shape)[is_ref]) + 0j
    pin[is_ref] = 1
    V0[~served] = 1.0 + 0.0j
    pin[~served] = 1
    return np.ascontiguousarray(V0), np.ascontiguousarray(pin)
