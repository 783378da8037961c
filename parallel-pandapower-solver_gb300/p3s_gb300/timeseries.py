"""Time-series injection matrix on the device (p3s/timeseries.py:36-141 ``build_sbus_matrix``).

The reference turns a pandapower time-series dict into the per-bus, per-step injection matrix
``Sbus`` (n_bus, T): the static base injection plus, per element and variable present in the
time series, ``sign / sn_mva * scaling * in_service * (value - base value)`` at the element's
bus (loads -1, sgen / gen +1; ``q_mvar`` to the imaginary part). This module keeps that
contract on array element tables (pandapower is not a dependency) and computes the matrix with
the ``gbpf_build_sbus`` kernel: the contributions are ordered bus-major with the element order
kept within a bus, as the reference orders them, and added in that order.
"""

from __future__ import annotations


import numpy as np

from . import _lib

ELEMENTS = ("load", "sgen", "gen")  # the reference's _TS_ELEMENTS, in its order


def contributions(n_bus: int, elements: dict, timeseries: dict, sn_mva: float = 1.0):
    """The reference's contribution list of ``build_sbus_matrix``.

    elements: name -> dict(bus=(n_el,) int (-1: unsupplied), p_mw=, q_mvar= (n_el,) base values,
    optional scaling=, in_service=); timeseries: (name, "p_mw" | "q_mvar") -> (n_el, T).
    Returns (T, ptr (n+1,) int64, row (K,) int32, coef, base (K,), imag (K,) uint8, series (R, T)).
    """
    names = [x for x in ELEMENTS if x in elements and len(elements[x]["bus"]) > 0]
    T = None
    for name in names:
        for var in ("p_mw", "q_mvar"):
            if (name, var) in timeseries:
                w = np.asarray(timeseries[(name, var)]).shape[1]
                T = w if T is None else min(T, w)
    if T is None:
        raise ValueError("no time-series data found for load/sgen/gen p_mw/q_mvar")
    sources, bus, row, src, coef, base, imag = [], [], [], [], [], [], []
    for name in names:
        el_tab = elements[name]
        lookup = np.asarray(el_tab["bus"], dtype=np.int64)
        el = np.nonzero(lookup >= 0)[0]
        sign = -1.0 if name == "load" else 1.0
        weight = np.ones(lookup.size)
        if "scaling" in el_tab:
            weight = weight * np.asarray(el_tab["scaling"], dtype=np.float64)
        if "in_service" in el_tab:
            weight = weight * np.asarray(el_tab["in_service"], dtype=bool)
        for var, is_imag in (("p_mw", False), ("q_mvar", True)):
            if (name, var) not in timeseries:
                continue
            base_v = np.asarray(el_tab[var], dtype=np.float64) if var in el_tab else np.zeros(lookup.size)
            sources.append(np.ascontiguousarray(np.asarray(timeseries[(name, var)])[:, :T], dtype=np.float64))
            bus.append(lookup[el])
            src.append(np.full(el.size, len(sources) - 1, dtype=np.int64))
            row.append(el)
            coef.append(sign / sn_mva * weight[el])
            base.append(base_v[el])
            imag.append(np.full(el.size, is_imag))
    bus_a = np.concatenate(bus)
    order = np.argsort(bus_a, kind="stable")
    ptr = np.zeros(n_bus + 1, dtype=np.int64)
    ptr[1:] = np.cumsum(np.bincount(bus_a, minlength=n_bus))
    offsets = np.cumsum([0] + [s.shape[0] for s in sources])
    src_a = np.concatenate(src)[order]
    row_a = (offsets[src_a] + np.concatenate(row)[order]).astype(np.int32)
    series = np.ascontiguousarray(np.concatenate(sources, axis=0)) if sources else np.zeros((0, T))
    return (T, ptr, row_a, np.ascontiguousarray(np.concatenate(coef)[order]),
            np.ascontiguousarray(np.concatenate(base)[order]),
            np.ascontiguousarray(np.concatenate(imag)[order], dtype=np.uint8), series)


def build_sbus(s0, ptr, row, coef, base, imag, series, T: int) -> np.ndarray:
    """(n, T) complex injections from a contribution list, computed on the device."""
    s0 = np.ascontiguousarray(s0, dtype=np.complex128)
    n = s0.shape[0]
    ptr = np.ascontiguousarray(ptr, dtype=np.int64)
    row = np.ascontiguousarray(row, dtype=np.int32)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    base = np.ascontiguousarray(base, dtype=np.float64)
    imag = np.ascontiguousarray(imag, dtype=np.uint8)
    series = np.ascontiguousarray(series, dtype=np.float64)
    if series.ndim != 2 or series.shape[1] != T or ptr.shape != (n + 1,):
        raise ValueError("build_sbus: series must be (R, T) and ptr (n + 1,)")
    out = np.empty((n, T), dtype=np.complex128)
    L = _lib.require_device()
    rc = L.gbpf_build_sbus(n, T, series.shape[0], _lib.cview(s0), _lib.i64(ptr), _lib.i32(row), _lib.d(coef),
                           _lib.d(base), _lib.u8(imag), _lib.d(series), _lib.cview(out))
    _lib.check(rc, "build_sbus")
    return out


def build_sbus_matrix(s_base, elements: dict, timeseries: dict, sn_mva: float = 1.0) -> np.ndarray:
    """``build_sbus_matrix`` on array element tables (see ``contributions``)."""
    s_base = np.ascontiguousarray(s_base, dtype=np.complex128)
    T, ptr, row, coef, base, imag, series = contributions(s_base.shape[0], elements, timeseries, sn_mva)
    return build_sbus(s_base, ptr, row, coef, base, imag, series, T)
