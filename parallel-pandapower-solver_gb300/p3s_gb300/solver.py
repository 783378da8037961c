"""Python owner of one device solver (C ABI of include/gbpf.h).

`GpuSolver` is the shared core behind both reference-facing surfaces
(``p3s_gb300.nr_klu`` and ``p3s_gb300.cuda.nr_polar_solver``): numpy arrays in, numpy
arrays out, every solve one launch of the persistent sm_103a Newton kernel.
"""

from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _lib
from .topology import jacobian_pattern, scalar_residual_order


def c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


class PinnedArray(np.ndarray):
    """numpy array over page-locked host memory (released with the array)."""

    def __array_finalize__(self, obj):
        if obj is not None:
            self._owner = getattr(obj, "_owner", None)


class _PinnedOwner:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        try:
            _lib.load().gbpf_host_free(self.ptr)
        except Exception:
            pass


def pinned_empty(shape, dtype) -> np.ndarray:
    """An uninitialised array in page-locked host memory (fast host <-> device copies)."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    ptr = _lib.load().gbpf_host_alloc(max(nbytes, 16))
    if not ptr:
        raise MemoryError(_lib.last_error())
    buf = (C.c_char * max(nbytes, 16)).from_address(ptr)
    a = np.frombuffer(buf, dtype=np.uint8, count=nbytes).view(dtype).reshape(shape).view(PinnedArray)
    a._owner = _PinnedOwner(ptr)
    return a


class _HostPool:
    """Page-locked blocks of dropped result arrays, kept for the next result of about the same
    size: a page-locked allocation costs milliseconds, and a fresh pageable array has its pages
    faulted in during the device-to-host copy. Holds at most `keep` bytes; the rest is freed."""

    def __init__(self, keep: int = 4 << 30):
        self.keep = keep
        self._free: list[tuple[int, int]] = []  # (bytes, address)
        self._held = 0
        self._lock = threading.Lock()

    def take(self, nbytes: int) -> tuple[int, int]:
        with self._lock:
            fit = [i for i, (nb, _) in enumerate(self._free) if nbytes <= nb <= 2 * nbytes]
            if fit:
                i = min(fit, key=lambda k: self._free[k][0])
                nb, ptr = self._free.pop(i)
                self._held -= nb
                return nb, ptr
        ptr = _lib.load().gbpf_host_alloc(nbytes)
        if not ptr:
            raise MemoryError(_lib.last_error())
        return nbytes, ptr

    def give(self, nbytes: int, ptr: int) -> None:
        with self._lock:
            if self._held + nbytes <= self.keep:
                self._free.append((nbytes, ptr))
                self._held += nbytes
                return
        _lib.load().gbpf_host_free(ptr)


_HOST_POOL = _HostPool()


class _PooledBlock:
    def __init__(self, nbytes, ptr):
        self.nbytes, self.ptr = nbytes, ptr

    def __del__(self):
        try:
            _HOST_POOL.give(self.nbytes, self.ptr)
        except Exception:
            pass


def pool_keep_at_least(nbytes: int) -> None:
    """Let the pool of page-locked result blocks hold at least `nbytes` of dropped blocks."""
    with _HOST_POOL._lock:
        _HOST_POOL.keep = max(_HOST_POOL.keep, int(nbytes))


def pooled_empty(shape, dtype) -> np.ndarray:
    """An uninitialised plain numpy array in page-locked host memory from a pool: the block
    goes back to the pool when the array and every view of it are gone (copies do not hold
    it)."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    nb, ptr = _HOST_POOL.take(max(nbytes, 16))
    buf = (C.c_char * nb).from_address(ptr)
    buf._block = _PooledBlock(nb, ptr)
    return np.frombuffer(buf, dtype=np.uint8, count=nbytes).view(dtype).reshape(shape)


class GpuSolver:
    """One grid topology resident on the device."""

    def __init__(self, Yp, Yj, Yx, pv, pq, cases_per_cta: int = 0, threads_per_cta: int = 0):
        L = _lib.require_device()
        self.Yp = np.ascontiguousarray(Yp, dtype=np.int32)
        self.Yj = np.ascontiguousarray(Yj, dtype=np.int32)
        self.Yx = c128(Yx)
        self.pv = np.ascontiguousarray(np.asarray(pv).ravel(), dtype=np.int32)
        self.pq = np.ascontiguousarray(np.asarray(pq).ravel(), dtype=np.int32)
        self.n = len(self.Yp) - 1
        self.nnz = len(self.Yj)
        if self.Yx.shape != (self.nnz,):
            raise ValueError("Yx must have one value per Ybus nonzero")
        h = L.gbpf_create_ex(self.n, _lib.i32(self.Yp), _lib.i32(self.Yj), _lib.cview(self.Yx), self.nnz,
                             _lib.i32(self.pv), len(self.pv), _lib.i32(self.pq), len(self.pq), int(cases_per_cta),
                             int(threads_per_cta))
        if not h:
            raise RuntimeError(_lib.last_error())
        self._h = h
        self._pattern = None
        self.chain_cap = 1.0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().gbpf_destroy(h)
            except Exception:
                pass
            self._h = None

    # -------------------------------------------------------------- facts
    @property
    def info(self) -> dict:
        o = _lib.Info()
        _lib.check(_lib.load().gbpf_get_info(self._h, C.byref(o)), "gbpf_get_info")
        return {f: getattr(o, f) for f, _ in o._fields_}

    @property
    def stats(self) -> dict:
        o = _lib.Stats()
        _lib.check(_lib.load().gbpf_get_stats(self._h, C.byref(o)), "gbpf_get_stats")
        return _lib.stats_dict(o)

    def last_mismatch(self, n_cases: int):
        """Final mismatch infinity norm (p.u.) of every case of the last synchronous solve, or
        None when the last call recorded none (an asynchronous call, or another case count)."""
        out = np.empty(int(n_cases))
        if _lib.load().gbpf_get_mismatch(self._h, _lib.d(out), int(n_cases)) != 0:
            return None
        return out

    def shape(self, units: int):
        """(threads per CTA, case slots per CTA) launched for a batch of `units` work items."""
        nt, g = C.c_int(), C.c_int()
        _lib.check(_lib.load().gbpf_get_shape(self._h, int(units), C.byref(nt), C.byref(g)), "gbpf_get_shape")
        return nt.value, g.value

    def prepare_shapes(self, max_cases_per_cta: int = 32):
        """Build the schedules of every CTA shape a launch may take (512 / 1,024 threads, up to
        ``max_cases_per_cta`` slots) now rather than on a later launch's critical path."""
        _lib.check(_lib.load().gbpf_prepare_shapes(self._h, int(max_cases_per_cta)), "gbpf_prepare_shapes")

    def set_shape(self, units: int, threads_per_cta: int, cases_per_cta: int):
        """Pin the CTA shape for batches of `units`' size class (0, 0 restores the rule)."""
        _lib.check(_lib.load().gbpf_set_shape(self._h, int(units), int(threads_per_cta), int(cases_per_cta)),
                   "gbpf_set_shape")

    def set_chain_cap(self, chain_cap: float):
        """Schedule knob of the factorization (gbpf_set_chain_cap): a level's pivot chain heavier
        than chain_cap x the level's mean work per worker is split over workers (0: never)."""
        _lib.check(_lib.load().gbpf_set_chain_cap(self._h, float(chain_cap)), "gbpf_set_chain_cap")
        self.chain_cap = float(chain_cap)

    def posmap(self) -> np.ndarray:
        out = np.empty(self.nnz, dtype=np.int32)
        _lib.check(_lib.load().gbpf_get_posmap(self._h, _lib.i32(out)))
        return out

    def row_of_bus(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.int32)
        _lib.check(_lib.load().gbpf_get_row_of_bus(self._h, _lib.i32(out)))
        return out

    @staticmethod
    def params(max_iter=30, tol=1e-8, line_search=True, precision="double", mixed_switch=1e-3, check_v0=False,
               pivot_ratio_double=1e-3, pivot_ratio_single=1e-3, vote_rule="gb300", polish=1e-3, vtol=1e-8,
               chord_tol=1e-8, shared_start=True, phase_timers=False, eager_jacobian=False):
        if precision not in ("double", "mixed"):
            raise ValueError(f"precision must be 'double' or 'mixed', got {precision!r}")
        return _lib.Params(int(max_iter), float(tol), int(bool(line_search)), 1 if precision == "mixed" else 0,
                           float(mixed_switch), int(bool(check_v0)), float(pivot_ratio_double),
                           float(pivot_ratio_single), 0 if vote_rule == "reference" else 1, float(polish),
                           float(vtol), float(chord_tol), int(bool(shared_start)), int(bool(phase_timers)),
                           int(bool(eager_jacobian)))

    def set_branches(self, f, t, stamp_pos, stamp, is_slack, gen_prio=None):
        """Branch table for outage cases: ends (m,), stamp CSR positions (m, 4) and values (m, 4)
        complex (Yff, Yft, Ytf, Ytt), slack flags (n,), re-slack priorities (n,) or None."""
        f = np.ascontiguousarray(f, dtype=np.int32)
        t = np.ascontiguousarray(t, dtype=np.int32)
        pos = np.ascontiguousarray(stamp_pos, dtype=np.int32)
        val = c128(stamp)
        sl = np.ascontiguousarray(is_slack, dtype=np.uint8)
        pr = None if gen_prio is None else np.ascontiguousarray(gen_prio, dtype=np.float64)
        m = len(f)
        if t.shape != (m,) or pos.shape != (m, 4) or val.shape != (m, 4) or sl.shape != (self.n,):
            raise ValueError("set_branches: f, t (m,), stamp_pos / stamp (m, 4), is_slack (n_bus,)")
        rc = _lib.load().gbpf_set_branches(self._h, m, _lib.i32(f), _lib.i32(t), _lib.i32(pos), _lib.cview(val),
                                           _lib.u8(sl), None if pr is None else _lib.d(pr))
        _lib.check(rc, "set_branches")
        self.branches = m

    def update_Y_from_branches(self, stamps, bus_shunt=None):
        """Ybus values summed on the device from branch stamps (m, 4) at the branch table's
        positions and bus shunts (n,) -- e.g. after tap changes (see ``ybus.branch_stamps``)."""
        st = c128(stamps)
        if st.shape != (getattr(self, "branches", -1), 4):
            raise ValueError("update_Y_from_branches: stamps must be (m, 4) for the branch table set")
        sh = None if bus_shunt is None else c128(np.asarray(bus_shunt).ravel())
        if sh is not None and sh.shape != (self.n,):
            raise ValueError("update_Y_from_branches: bus_shunt must be (n_bus,)")
        rc = _lib.load().gbpf_update_Y_from_branches(self._h, _lib.cview(st), None if sh is None else _lib.cview(sh))
        _lib.check(rc, "update_Y_from_branches")
        Yx = np.empty(self.nnz, dtype=np.complex128)
        _lib.check(_lib.load().gbpf_get_Y(self._h, _lib.cview(Yx)), "gbpf_get_Y")
        self.Yx = Yx

    # -------------------------------------------------------------- values
    def update_Y(self, Yx):
        Yx = c128(Yx)
        if Yx.shape != (self.nnz,):
            raise ValueError("update_Y: nnz mismatch (topology changed; rebuild the solver)")
        _lib.check(_lib.load().gbpf_update_Y(self._h, _lib.cview(Yx), self.nnz), "update_Y")
        self.Yx = Yx

    # -------------------------------------------------------------- solves
    def solve_batch(self, S, V0, p: _lib.Params):
        """S (n, T) or (n,) with T given by V0; V0 (n,) or (n, T)."""
        S = c128(S)
        V0 = c128(V0)
        T = S.shape[1] if S.ndim == 2 else V0.shape[1]
        V = np.empty((self.n, T), dtype=np.complex128)
        it = np.empty(T, dtype=np.int32)
        cv = np.empty(T, dtype=np.uint8)
        rc = _lib.load().gbpf_solve_batch(self._h, T, _lib.cview(S), int(S.ndim == 2), _lib.cview(V0),
                                          int(V0.ndim == 2), C.byref(p), _lib.cview(V), _lib.i32(it), _lib.u8(cv))
        _lib.check(rc, "solve_batch")
        return {"V": V, "iterations": it, "converged": cv.astype(bool)}

    def solve_lanes(self, S, V0, offsets, p: _lib.Params, out=None):
        """``out`` = (V, iterations, converged) caller-owned result arrays (e.g. pinned)."""
        S = c128(S)
        V0 = c128(V0).ravel()
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        T = S.shape[1]
        K = len(off) - 1
        if out is None:
            V = np.empty((self.n, T), dtype=np.complex128)
            it = np.empty(T, dtype=np.int32)
            cv = np.empty(T, dtype=np.uint8)
        else:
            V, it, cv = out
        rc = _lib.load().gbpf_solve_lanes(self._h, T, _lib.cview(S), _lib.cview(V0), K, _lib.i64(off), C.byref(p),
                                          _lib.cview(V), _lib.i32(it), _lib.u8(cv))
        _lib.check(rc, "solve_lanes")
        return {"V": V, "iterations": it, "converged": cv.view(bool) if out is not None else cv.astype(bool)}

    def solve_lanes_async(self, slot: int, S, V0, offsets, p: _lib.Params, out):
        """Enqueue ``solve_lanes`` in `slot` and return at once; the arrays (use ``pinned_empty``
        for S and the outputs) must stay alive until ``wait(slot)``. out = (V, iterations,
        converged) caller-owned result arrays."""
        V, it, cv = out
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        if not (S.flags.c_contiguous and S.dtype == np.complex128):
            raise ValueError("solve_lanes_async: S must be a C-contiguous complex128 array")
        V0 = c128(V0).ravel()
        self._async_keep = getattr(self, "_async_keep", {})
        self._async_keep[slot] = (S, V0, off, V, it, cv)
        rc = _lib.load().gbpf_solve_lanes_async(self._h, int(slot), S.shape[1], _lib.cview(S), _lib.cview(V0),
                                                len(off) - 1, _lib.i64(off), C.byref(p), _lib.cview(V), _lib.i32(it),
                                                _lib.u8(cv))
        _lib.check(rc, "solve_lanes_async")

    def wait(self, slot: int):
        """Wait for the call in `slot`; its results are in the arrays handed to it."""
        rc = _lib.load().gbpf_solve_wait(self._h, int(slot))
        keep = getattr(self, "_async_keep", {}).pop(slot, None)
        _lib.check(rc, "solve_wait")
        return keep

    def solve_lanes_device(self, dS: int, dV0: int, doff: int, T: int, K: int, p: _lib.Params, dV: int, dit: int,
                           dcv: int):
        """Device-pointer variant (inputs already resident); pointers as integers."""
        rc = _lib.load().gbpf_solve_lanes_device(self._h, T, dS, dV0, K, doff, C.byref(p), dV, dit, dcv)
        _lib.check(rc, "solve_lanes_device")

    def solve_contingency(self, S, V0, pin, p: _lib.Params, Yd=None, stamps=None):
        """S (n,), V0 (n, L), pin (n, L) or None; per-case Ybus: Yd (nnz, L) complex or
        stamps = (ptr (L+1,), k (E,), val (E,) complex) subtracted from the base values."""
        S = c128(np.asarray(S).ravel())
        V0 = c128(V0)
        L = V0.shape[1]
        pin_a = None if pin is None else np.ascontiguousarray(pin, dtype=np.uint8)
        V = np.empty((self.n, L), dtype=np.complex128)
        it = np.empty(L, dtype=np.int32)
        cv = np.empty(L, dtype=np.uint8)
        Ydp = None
        sp_ = sk = sv = None
        if Yd is not None:
            Yd = c128(Yd)
            Ydp = _lib.cview(Yd)
        elif stamps is not None:
            ptr, k, val = stamps
            ptr = np.ascontiguousarray(ptr, dtype=np.int32)
            k = np.ascontiguousarray(k, dtype=np.int32)
            val = c128(val)
            sp_, sk, sv = _lib.i32(ptr), _lib.i32(k), _lib.cview(val)
        rc = _lib.load().gbpf_solve_contingency(self._h, L, _lib.cview(S), _lib.cview(V0),
                                                None if pin_a is None else _lib.u8(pin_a), Ydp, sp_, sk, sv,
                                                C.byref(p), _lib.cview(V), _lib.i32(it), _lib.u8(cv))
        _lib.check(rc, "solve_batch_contingency")
        return {"V": V, "iterations": it, "converged": cv.astype(bool)}

    def dc_start(self, Pinj, V0, dc_stamps=None):
        """DC start voltage (``dc_initial_voltage``): DC angles at every non-slack bus with V0's
        magnitudes; V0 itself when the DC system is singular. Pinj (n,) or (n, T): one or T cases
        (time steps, scenarios) solved with ONE factorization of B. dc_stamps: (m, 4) complex DC
        branch stamps of the reference's models (``ybus.branch_stamps`` of the ``ys_dc`` two-ports,
        at the positions of ``set_branches``) -- B is then the reference's Bbus; None: B from the
        Ybus. Returns (V, used) -- V and used shaped like Pinj's cases (used: DC angles taken)."""
        P = np.asarray(Pinj, dtype=np.float64)
        one = P.ndim == 1
        P = np.ascontiguousarray(P.reshape(self.n, -1) if P.size else P)
        V0 = c128(np.asarray(V0).ravel())
        if P.ndim != 2 or P.shape[0] != self.n or P.shape[1] < 1 or V0.shape != (self.n,):
            raise ValueError("dc_start: Pinj must be (n_bus,) or (n_bus, T) and V0 (n_bus,)")
        T = P.shape[1]
        st = None
        if dc_stamps is not None:
            st = c128(dc_stamps)
            if st.shape != (getattr(self, "branches", -1), 4):
                raise ValueError("dc_start: dc_stamps must be (n_branch, 4) complex (after set_branches)")
        out = np.empty((self.n, T), dtype=np.complex128)
        used = np.empty(T, dtype=np.uint8)
        rc = _lib.load().gbpf_dc_start_batch(self._h, T, _lib.d(P), _lib.cview(V0),
                                             None if st is None else _lib.cview(st), _lib.cview(out), _lib.u8(used))
        if rc < 0:
            raise RuntimeError(_lib.last_error())
        if one:
            return out[:, 0], bool(used[0])
        return out, used.astype(bool)

    # -------------------------------------------------------------- Jacobian
    def eval_blocks(self, S, V, pin=None):
        """Device Jacobian blocks (n_blocks, 4) and residual (n_var_bus, 2) at one voltage."""
        S = c128(np.asarray(S).ravel())
        V = c128(np.asarray(V).ravel())
        info = self.info
        blk = np.empty((info["n_blocks"], 4), dtype=np.float64)
        R = np.empty((max(info["n_var_bus"], 1), 2), dtype=np.float64)
        pin_a = None if pin is None else np.ascontiguousarray(pin, dtype=np.uint8)
        rc = _lib.load().gbpf_eval_jacobian(self._h, _lib.cview(S), _lib.cview(V),
                                            None if pin_a is None else _lib.u8(pin_a), _lib.d(blk), _lib.d(R))
        _lib.check(rc, "eval_jacobian")
        return blk, R[: info["n_var_bus"]]

    def debug_J(self, S, V):
        """The reference's debug_J result (CSC Jp, Ji, Jx, m) from the device Jacobian, plus
        the mismatch F = S(V) - S in the reference's row order."""
        if self._pattern is None:
            self._pattern = jacobian_pattern(self.Yp, self.Yj, self.pv, self.pq)
        Jp, Ji, sk, sb, m = self._pattern
        blk, R = self.eval_blocks(S, V)
        pm = self.posmap()
        Jx = blk[pm[sk], sb]
        rob = self.row_of_bus()
        row_p, row_q = scalar_residual_order(self.pv, self.pq, self.n)
        F = np.zeros(m)
        bus = np.nonzero(row_p >= 0)[0]
        F[row_p[bus]] = -R[rob[bus], 0]
        bq = np.nonzero(row_q >= 0)[0]
        F[row_q[bq]] = -R[rob[bq], 1]
        return {"Jp": Jp, "Ji": Ji, "Jx": Jx, "m": m, "F": F}
