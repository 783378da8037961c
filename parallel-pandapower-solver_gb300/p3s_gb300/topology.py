"""Host-side Jacobian pattern in the reference's scalar layout.

The device works on 2x2 bus blocks; callers of the reference see the scalar Jacobian of
``nr_klu.cpp:230-285`` (CSC; columns: angle of every pv/pq bus, then magnitude of every
pq bus; in a column the P rows come before the Q rows, each in Ybus row order; a
nonzero's value is one of the four derivative blocks of one Ybus nonzero, recorded as
``(src_k, src_block)`` with block ids 0=dP/dVa, 1=dP/dVm, 2=dQ/dVa, 3=dQ/dVm). This module
rebuilds that layout so a device block array can be handed out as the reference's
``debug_J`` result.
"""

from __future__ import annotations

import numpy as np


def jacobian_pattern(Yp, Yj, pv, pq):
    """(Jp, Ji, src_k, src_block, m) of the reference's CSC Jacobian pattern."""
    Yp = np.asarray(Yp, dtype=np.int64)
    Yj = np.asarray(Yj, dtype=np.int64)
    pv = np.asarray(pv, dtype=np.int64).ravel()
    pq = np.asarray(pq, dtype=np.int64).ravel()
    n = len(Yp) - 1
    pvpq = np.concatenate([pv, pq])
    npvpq = len(pvpq)
    m = npvpq + len(pq)
    pvpq_pos = np.full(n, -1, dtype=np.int64)
    pvpq_pos[pvpq] = np.arange(npvpq)
    pq_pos = np.full(n, -1, dtype=np.int64)
    pq_pos[pq] = np.arange(len(pq))
    row = np.repeat(np.arange(n), np.diff(Yp))
    k = np.arange(len(Yj))
    order = np.lexsort((row, Yj))
    cs, rs, ks = Yj[order], row[order], k[order]
    cptr = np.searchsorted(cs, np.arange(n + 1))
    Ji, sk, sb = [], [], []
    Jp = np.zeros(m + 1, dtype=np.int32)
    cols = [(b, False) for b in pvpq] + [(b, True) for b in pq]
    tot = 0
    for c, (bus, vm) in enumerate(cols):
        r = rs[cptr[bus]:cptr[bus + 1]]
        kk = ks[cptr[bus]:cptr[bus + 1]]
        mp = pvpq_pos[r] >= 0
        mq = pq_pos[r] >= 0
        Ji.append(pvpq_pos[r[mp]])
        sk.append(kk[mp])
        sb.append(np.full(mp.sum(), 1 if vm else 0))
        Ji.append(npvpq + pq_pos[r[mq]])
        sk.append(kk[mq])
        sb.append(np.full(mq.sum(), 3 if vm else 2))
        tot += int(mp.sum() + mq.sum())
        Jp[c + 1] = tot
    cat = lambda a: np.concatenate(a).astype(np.int32) if a else np.zeros(0, np.int32)  # noqa: E731
    return Jp, cat(Ji), cat(sk), cat(sb), m


def scalar_residual_order(pv, pq, n):
    """(row_p, row_q): the reference's mismatch row of each bus's P / Q equation (-1: none)."""
    pv = np.asarray(pv, dtype=np.int64).ravel()
    pq = np.asarray(pq, dtype=np.int64).ravel()
    pvpq = np.concatenate([pv, pq])
    row_p = np.full(n, -1, dtype=np.int64)
    row_p[pvpq] = np.arange(len(pvpq))
    row_q = np.full(n, -1, dtype=np.int64)
    row_q[pq] = len(pvpq) + np.arange(len(pq))
    return row_p, row_q
