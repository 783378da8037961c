"""ctypes front end of the CPU oracle (``liboracle.so``, built from nr_oracle.cpp).

TEST INFRASTRUCTURE ONLY. The oracle restates the reference's ``p3s/cpp/nr_klu.cpp``
(see nr_oracle.cpp); this module gives it the reference's Python call surface
(``nr_klu.cpp:1315-1376``): ``Solver(Yp, Yj, Yx, pv, pq)`` with ``solve``, ``solve_batch``,
``solve_batch_contingency``, ``update_Y``, ``lean_active``, plus ``solve_single`` and
``debug_J``. Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use it.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_P = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_bp = C.POINTER(C.c_ubyte)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from oracle.build import build_oracle

            build_oracle()
        L = C.CDLL(LIB_PATH)
        L.oracle_create.restype = _P
        L.oracle_create.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, _ip, C.c_int, _ip, C.c_int, C.c_char_p, C.c_int]
        L.oracle_destroy.argtypes = [_P]
        L.oracle_lean_active.argtypes = [_P]
        L.oracle_sizes.argtypes = [_P, _ip, _ip]
        L.oracle_update_Y.argtypes = [_P, _dp, C.c_int]
        L.oracle_solve_batch.argtypes = [_P, _dp, C.c_int, _dp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                         _dp, _ip, _bp, C.c_char_p, C.c_int]
        L.oracle_solve_batch_contingency.argtypes = [_P, _dp, _dp, C.c_int, _dp, _dp, _bp, C.c_int, C.c_double,
                                                     C.c_int, C.c_int, _dp, _ip, _bp, C.c_char_p, C.c_int]
        L.oracle_debug_J.argtypes = [_P, _dp, _dp, _ip, _ip, _dp, _dp]
        L.oracle_last_paths.argtypes = [_P, _ip, C.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _b(a):
    return a.ctypes.data_as(_bp)


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


class Solver:
    """The oracle with ``nr_klu.Solver``'s signature (``nr_klu.cpp:964-1313``)."""

    def __init__(self, Yp, Yj, Yx, pv, pq, ordering: int = 0, btf: int = 0):
        self.Yp = np.ascontiguousarray(Yp, dtype=np.int32)
        self.Yj = np.ascontiguousarray(Yj, dtype=np.int32)
        Yx = _c128(Yx)
        pv = np.ascontiguousarray(pv, dtype=np.int32)
        pq = np.ascontiguousarray(pq, dtype=np.int32)
        self.n = len(self.Yp) - 1
        self.nnz = len(self.Yj)
        err = C.create_string_buffer(512)
        self._h = lib().oracle_create(self.n, _i(self.Yp), _i(self.Yj), _d(Yx.view(np.float64)), self.nnz, _i(pv),
                                      len(pv), _i(pq), len(pq), err, 512)
        if not self._h:
            raise RuntimeError(err.value.decode() or "oracle_create failed")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.oracle_destroy(h)
            self._h = None

    def last_paths(self):
        """Per column of the last batch call: 0 solved on the frozen (lean) pivot order throughout,
        1 a lean refactorization failed its pivot check and the column went on with pivoting
        LU (nr_klu.cpp:610-652), 2 re-run from its start on pivoting LU (nr_klu.cpp:845-857)."""
        n = lib().oracle_last_paths(self._h, None, 0)
        out = np.zeros(n, dtype=np.int32)
        lib().oracle_last_paths(self._h, _i(out), n)
        return out

    @property
    def lean_active(self) -> bool:
        return bool(lib().oracle_lean_active(self._h))

    def update_Y(self, Yx):
        Yx = _c128(Yx)
        if Yx.shape[0] != self.nnz or lib().oracle_update_Y(self._h, _d(Yx.view(np.float64)), self.nnz) != 0:
            raise RuntimeError("update_Y: nnz mismatch (topology changed; rebuild Solver)")

    def solve_batch(self, Sbus, V0, max_iter: int = 30, tol: float = 1e-8, n_threads: int = 0,
                    line_search: bool = True):
        Sbus = _c128(Sbus)
        if Sbus.ndim != 2:
            raise RuntimeError("solve_batch: Sbus must be 2-D (n, T)")
        if Sbus.shape[0] != self.n:
            raise RuntimeError("solve_batch: Sbus rows must equal n_bus")
        T = Sbus.shape[1]
        if T == 0:
            raise RuntimeError("solve_batch: T (time steps) must be > 0")
        if max_iter <= 0:
            raise RuntimeError("solve_batch: max_iter must be > 0")
        if tol <= 0.0:
            raise RuntimeError("solve_batch: tol must be > 0")
        if n_threads < 0:
            raise RuntimeError("solve_batch: n_threads must be >= 0")
        V0 = _c128(V0)
        per_col = V0.ndim == 2
        if per_col and V0.shape != (self.n, T):
            raise RuntimeError("solve_batch: V0 (n,T) shape mismatch")
        if not per_col and V0.shape[0] != self.n:
            raise RuntimeError("solve_batch: V0 (n,) length mismatch")
        V = np.empty((self.n, T), dtype=np.complex128)
        it = np.empty(T, dtype=np.int32)
        cv = np.empty(T, dtype=np.uint8)
        err = C.create_string_buffer(512)
        rc = lib().oracle_solve_batch(self._h, _d(Sbus.view(np.float64)), T, _d(V0.view(np.float64)), int(per_col),
                                      int(max_iter), float(tol), int(n_threads), int(bool(line_search)),
                                      _d(V.view(np.float64)), _i(it), _b(cv), err, 512)
        if rc != 0:
            raise RuntimeError("solve_batch: " + err.value.decode())
        return {"V": V, "iterations": it, "converged": cv.astype(bool)}

    def solve(self, Sbus, V0, max_iter: int = 30, tol: float = 1e-8, line_search: bool = True):
        r = self.solve_batch(_c128(Sbus)[:, None], _c128(V0), max_iter, tol, 1, line_search)
        return {"V": r["V"][:, 0].copy(), "iterations": int(r["iterations"][0]), "converged": bool(r["converged"][0])}

    def solve_batch_contingency(self, Yx_mag, Yx_ang, Sbus, V0, pin, max_iter: int = 30, tol: float = 1e-8,
                                n_threads: int = 0, line_search: bool = True):
        Ym = np.ascontiguousarray(Yx_mag, dtype=np.float64)
        Ya = np.ascontiguousarray(Yx_ang, dtype=np.float64)
        if Ym.ndim != 2 or Ya.ndim != 2:
            raise RuntimeError("solve_batch_contingency: Yx_mag/ang must be 2-D (nnz, L)")
        if Ym.shape[0] != self.nnz:
            raise RuntimeError("solve_batch_contingency: Yx rows must equal Ybus nnz")
        L = Ym.shape[1]
        if Ya.shape != (self.nnz, L):
            raise RuntimeError("solve_batch_contingency: Yx_mag/ang shape mismatch")
        V0 = _c128(V0)
        if V0.shape != (self.n, L):
            raise RuntimeError("solve_batch_contingency: V0 must be (n, L)")
        pin = np.ascontiguousarray(pin, dtype=np.uint8)
        if pin.shape != (self.n, L):
            raise RuntimeError("solve_batch_contingency: pin must be (n, L)")
        S = _c128(np.asarray(Sbus).ravel())
        V = np.empty((self.n, L), dtype=np.complex128)
        it = np.empty(L, dtype=np.int32)
        cv = np.empty(L, dtype=np.uint8)
        err = C.create_string_buffer(512)
        rc = lib().oracle_solve_batch_contingency(self._h, _d(Ym), _d(Ya), L, _d(S.view(np.float64)),
                                                  _d(V0.view(np.float64)), _b(pin), int(max_iter), float(tol),
                                                  int(n_threads), int(bool(line_search)), _d(V.view(np.float64)),
                                                  _i(it), _b(cv), err, 512)
        if rc != 0:
            raise RuntimeError("solve_batch_contingency: " + err.value.decode())
        return {"V": V, "iterations": it, "converged": cv.astype(bool)}

    def debug_J_at(self, Sbus, V0):
        m = C.c_int()
        nz = C.c_int()
        lib().oracle_sizes(self._h, C.byref(m), C.byref(nz))
        Jp = np.empty(m.value + 1, dtype=np.int32)
        Ji = np.empty(nz.value, dtype=np.int32)
        Jx = np.empty(nz.value, dtype=np.float64)
        F = np.empty(m.value, dtype=np.float64)
        S = _c128(Sbus)
        V = _c128(V0)
        lib().oracle_debug_J(self._h, _d(S.view(np.float64)), _d(V.view(np.float64)), _i(Jp), _i(Ji), _d(Jx), _d(F))
        return {"Jp": Jp, "Ji": Ji, "Jx": Jx, "m": m.value, "F": F}


def solve_single(Yp, Yj, Yx, Sbus, V0, pv, pq, max_iter=30, tol=1e-8, ordering=0, btf=0, line_search=True):
    r = Solver(Yp, Yj, Yx, pv, pq).solve(Sbus, V0, max_iter, tol, line_search)
    return r


def debug_J(Yp, Yj, Yx, Sbus, V0, pv, pq):
    d = Solver(Yp, Yj, Yx, pv, pq).debug_J_at(Sbus, V0)
    d.pop("F")
    return d


def solve_lanes(solver: Solver, Sbus, V0, offsets, max_iter=30, tol=1e-8, n_threads=0, line_search=True):
    """Warm-start lanes replayed wave by wave: hour ``offsets[l] + w`` of lane ``l`` starts
    from the converged voltage of hour ``offsets[l] + w - 1`` (from ``V0`` for the lane's
    first hour, and after a non-converged hour)."""
    Sbus = _c128(Sbus)
    n, T = Sbus.shape
    K = len(offsets) - 1
    V = np.empty((n, T), dtype=np.complex128)
    it = np.zeros(T, dtype=np.int32)
    cv = np.zeros(T, dtype=bool)
    V0 = _c128(V0)
    cur = np.repeat(V0[:, None], K, axis=1)
    length = np.diff(offsets)
    for w in range(int(length.max())):
        lanes_w = np.nonzero(length > w)[0]
        cols = offsets[lanes_w] + w
        r = solver.solve_batch(np.ascontiguousarray(Sbus[:, cols]), np.ascontiguousarray(cur[:, lanes_w]), max_iter,
                               tol, n_threads, line_search)
        V[:, cols] = r["V"]
        it[cols] = r["iterations"]
        cv[cols] = r["converged"]
        ok = r["converged"]
        cur[:, lanes_w[ok]] = r["V"][:, ok]
        cur[:, lanes_w[~ok]] = V0[:, None]
    return {"V": V, "iterations": it, "converged": cv}
