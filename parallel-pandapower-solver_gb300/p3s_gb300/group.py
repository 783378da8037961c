"""Several topologies in one launch of the persistent Newton kernel (include/gbpf.h group API).

A ``GpuGroup`` owns a stream, scratch and staging buffers; ``solve`` takes one job per
topology (a ``GpuSolver`` and its cases) and runs them all in ONE launch, largest job first,
so grids of uneven size and the requests of a serving loop share the device instead of
queueing behind each other. Per case the arithmetic is the single-topology solve's, so
every result equals the one ``GpuSolver`` returns for the same case (bit for bit).
No reference counterpart: the reference solves one topology per call.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .solver import GpuSolver, c128, pooled_empty


@dataclass
class GroupJob:
    """One topology's cases. S: (n, T) or (n,) with T from V0; V0: (n,) or (n, T); pin: (n, T)
    or None; stamps: (ptr (T+1,), k, val) outage stamps subtracted from the base Ybus, or None;
    outages: (ptr (T+1,), idx) branch outages of every case, islanded on the device (the
    solver's branch table must be set, S and V0 are (n,)), or None."""

    solver: GpuSolver
    S: np.ndarray
    V0: np.ndarray
    n_cases: int = 0
    pin: np.ndarray | None = None
    stamps: tuple | None = None
    cases_per_cta: int = 0
    outages: tuple | None = None
    reslack: bool = True


class GpuGroup:
    def __init__(self):
        L = _lib.require_device()
        h = L.gbpf_group_create()
        if not h:
            raise RuntimeError(_lib.last_error())
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().gbpf_group_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_shape(self, threads_per_cta: int = 0, slot_budget: int = 0):
        """Threads per CTA of later launches (0: by batch size) and the variable buses x case
        slots a CTA may hold per job (0: 16,384)."""
        _lib.check(_lib.load().gbpf_group_set_shape(self._h, int(threads_per_cta), int(slot_budget)),
                   "gbpf_group_set_shape")

    @property
    def stats(self) -> dict:
        o = _lib.Stats()
        _lib.check(_lib.load().gbpf_group_stats(self._h, C.byref(o)), "gbpf_group_stats")
        return _lib.stats_dict(o)

    def solve(self, jobs: list[GroupJob], params: _lib.Params, pinned_out: bool = False) -> list[dict]:
        """One launch over `jobs`; per job a dict of V (n, T), iterations, converged and, for
        outage jobs, served (n, T). pinned_out: V and served of 1 MB or more in pooled
        page-locked host memory (a direct copy from the device; the block is reused once the
        arrays are dropped)."""

        def empty(shape, dtype):
            big = pinned_out and shape[0] * shape[1] * np.dtype(dtype).itemsize >= 1 << 20
            return pooled_empty(shape, dtype) if big else np.empty(shape, dtype=dtype)

        arr = (_lib.Job * len(jobs))()
        keep = []
        outs = []
        for i, jb in enumerate(jobs):
            n = jb.solver.n
            S = c128(jb.S)
            V0 = c128(jb.V0)
            T = jb.n_cases or (S.shape[1] if S.ndim == 2 else (V0.shape[1] if V0.ndim == 2 else 1))
            if S.shape not in ((n, T), (n,)) or V0.shape not in ((n, T), (n,)):
                raise ValueError(f"job {i}: S / V0 must be (n_bus, T) or (n_bus,)")
            V = empty((n, T), dtype=np.complex128)
            it = np.empty(T, dtype=np.int32)
            cv = np.empty(T, dtype=np.uint8)
            J = arr[i]
            J.solver = jb.solver._h
            J.n_cases = T
            J.S = S.ctypes.data
            J.s_per_col = int(S.ndim == 2)
            J.V0 = V0.ctypes.data
            J.v0_per_col = int(V0.ndim == 2)
            keep += [S, V0]
            if jb.pin is not None:
                pin = np.ascontiguousarray(jb.pin, dtype=np.uint8)
                if pin.shape != (n, T):
                    raise ValueError(f"job {i}: pin must be (n_bus, T)")
                J.pin = pin.ctypes.data
                keep.append(pin)
            if jb.stamps is not None:
                ptr, k, val = jb.stamps
                ptr = np.ascontiguousarray(ptr, dtype=np.int32)
                k = np.ascontiguousarray(k, dtype=np.int32)
                val = c128(val)
                if ptr.shape != (T + 1,):
                    raise ValueError(f"job {i}: stamp pointers must be (T + 1,)")
                J.st_ptr, J.st_k, J.st_val = ptr.ctypes.data, k.ctypes.data, val.ctypes.data
                keep += [ptr, k, val]
            J.V, J.iterations, J.converged = V.ctypes.data, it.ctypes.data, cv.ctypes.data
            J.cases_per_cta = int(jb.cases_per_cta)
            if jb.outages is not None:
                optr, oidx = jb.outages
                optr = np.ascontiguousarray(optr, dtype=np.int32)
                oidx = np.ascontiguousarray(oidx, dtype=np.int32)
                if optr.shape != (T + 1,):
                    raise ValueError(f"job {i}: outage pointers must be (T + 1,)")
                J.out_ptr, J.out_idx, J.reslack = optr.ctypes.data, oidx.ctypes.data, int(bool(jb.reslack))
                keep += [optr, oidx]
                sv = empty((n, T), dtype=np.uint8)  # the device islanding's served mask
                J.served = sv.ctypes.data
            else:
                sv = None
            outs.append((V, it, cv, sv))
        rc = _lib.load().gbpf_group_solve(self._h, len(jobs), arr, C.byref(params))
        _lib.check(rc, "group_solve")
        res = []
        for V, it, cv, sv in outs:
            r = {"V": V, "iterations": it, "converged": cv.view(bool)}
            if sv is not None:
                r["served"] = sv.view(bool)
            res.append(r)
        return res
