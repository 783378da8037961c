"""Drop-in for the reference's ``p3s.cpp.nr_klu`` pybind11 module (nr_klu.cpp:1315-1376).

Same entry points, keyword arguments, dtypes, result keys and error messages; the solves
run on the GB300 (one persistent-kernel launch per call) in double precision. A caller
switches with ``from p3s_gb300 import nr_klu``.

Differences, by design:
* ``n_threads`` is validated like the reference and otherwise has no effect (the device
  runs every column in parallel); ``openmp`` is False for the same reason.
* ``ordering`` / ``btf`` (KLU options) are accepted and ignored: the device uses its own
  fill-reducing order on 2x2 bus blocks.
* A column whose frozen-order factorization fails the pivot check is reported not
  converged; the reference re-solves such a column with KLU's pivoting factorization
  (nr_klu.cpp:845-857). No such column occurs on the benchmark grids (checked in tests).
"""

from __future__ import annotations

import time

import numpy as np

from .solver import GpuSolver, c128

openmp = False


def _err(msg):
    return RuntimeError(msg)


class Solver:
    """``nr_klu.Solver(Yp, Yj, Yx, pv, pq, ordering=0, btf=0)`` (nr_klu.cpp:964-1313)."""

    def __init__(self, Yp, Yj, Yx, pv, pq, ordering: int = 0, btf: int = 0):
        self._s = GpuSolver(Yp, Yj, Yx, pv, pq)
        self.n = self._s.n
        self.nnz = self._s.nnz

    @property
    def lean_active(self) -> bool:
        return True

    def update_Y(self, Yx):
        Yx = c128(Yx)
        if Yx.shape[0] != self.nnz:
            raise _err("update_Y: nnz mismatch (topology changed; rebuild Solver)")
        self._s.update_Y(Yx)

    def solve(self, Sbus, V0, max_iter: int = 30, tol: float = 1e-8, line_search: bool = True):
        Sbus = c128(Sbus).ravel()
        V0 = c128(V0).ravel()
        if Sbus.shape[0] != self.n or V0.shape[0] != self.n:
            raise _err("solve: Sbus / V0 length must equal n_bus")
        p = GpuSolver.params(max_iter, tol, line_search)
        r = self._s.solve_batch(Sbus[:, None], V0, p)
        return {"V": r["V"][:, 0].copy(), "iterations": int(r["iterations"][0]), "converged": bool(r["converged"][0])}

    def solve_batch(self, Sbus, V0, max_iter: int = 30, tol: float = 1e-8, n_threads: int = 0,
                    line_search: bool = True):
        Sbus = c128(Sbus)
        if Sbus.ndim != 2:
            raise _err("solve_batch: Sbus must be 2-D (n, T)")
        if Sbus.shape[0] != self.n:
            raise _err("solve_batch: Sbus rows must equal n_bus")
        T = Sbus.shape[1]
        if T == 0:
            raise _err("solve_batch: T (time steps) must be > 0")
        if max_iter <= 0:
            raise _err("solve_batch: max_iter must be > 0")
        if tol <= 0.0:
            raise _err("solve_batch: tol must be > 0")
        if n_threads < 0:
            raise _err("solve_batch: n_threads must be >= 0")
        V0 = c128(V0)
        if V0.ndim == 2:
            if V0.shape != (self.n, T):
                raise _err("solve_batch: V0 (n,T) shape mismatch")
        elif V0.shape[0] != self.n:
            raise _err("solve_batch: V0 (n,) length mismatch")
        p = GpuSolver.params(max_iter, tol, line_search, check_v0=True)
        return self._s.solve_batch(Sbus, V0, p)

    def solve_batch_contingency(self, Yx_mag, Yx_ang, Sbus, V0, pin, max_iter: int = 30, tol: float = 1e-8,
                                n_threads: int = 0, line_search: bool = True):
        Ym = np.asarray(Yx_mag, dtype=np.float64)
        Ya = np.asarray(Yx_ang, dtype=np.float64)
        if Ym.ndim != 2 or Ya.ndim != 2:
            raise _err("solve_batch_contingency: Yx_mag/ang must be 2-D (nnz, L)")
        if Ym.shape[0] != self.nnz:
            raise _err("solve_batch_contingency: Yx rows must equal Ybus nnz")
        L = Ym.shape[1]
        if Ya.shape != (self.nnz, L):
            raise _err("solve_batch_contingency: Yx_mag/ang shape mismatch")
        V0 = c128(V0)
        if V0.ndim != 2 or V0.shape != (self.n, L):
            raise _err("solve_batch_contingency: V0 must be (n, L)")
        pin = np.ascontiguousarray(pin, dtype=np.uint8)
        if pin.ndim != 2 or pin.shape != (self.n, L):
            raise _err("solve_batch_contingency: pin must be (n, L)")
        Yd = Ym * np.exp(1j * Ya)
        p = GpuSolver.params(max_iter, tol, line_search)
        return self._s.solve_contingency(Sbus, V0, pin, p, Yd=Yd)

    def debug_J_at(self, Sbus, V0):
        d = self._s.debug_J(Sbus, V0)
        d.pop("F")
        return d


def solve_single(Yp, Yj, Yx, Sbus, V0, pv, pq, max_iter: int = 30, tol: float = 1e-8, ordering: int = 0,
                 btf: int = 0, line_search: bool = True):
    """``nr_klu.solve_single`` (nr_klu.cpp:868-951)."""
    t0 = time.perf_counter()
    s = Solver(Yp, Yj, Yx, pv, pq, ordering, btf)
    t1 = time.perf_counter()
    r = s.solve(Sbus, V0, max_iter, tol, line_search)
    t2 = time.perf_counter()
    return {
        "V": r["V"],
        "iterations": r["iterations"],
        "converged": r["converged"],
        "t_setup_ms": (t1 - t0) * 1e3,
        "t_solve_ms": (t2 - t1) * 1e3,
        "t_assemble_ms": 0.0,
        "profiled": False,
    }


def debug_J(Yp, Yj, Yx, Sbus, V0, pv, pq):
    """``nr_klu.debug_J`` (nr_klu.cpp:1332-1342): the Jacobian (CSC) at V0."""
    return Solver(Yp, Yj, Yx, pv, pq).debug_J_at(Sbus, V0)
