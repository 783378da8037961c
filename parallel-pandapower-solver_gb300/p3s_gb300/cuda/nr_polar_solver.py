"""Drop-in for the reference's ``PolarNewtonSolverCUDA`` (p3s/cuda/nr_polar_solver.py:279-596).

Same constructor, attributes and methods; the batch runs as one launch of the persistent
sm_103a Newton kernel (no memory chunking, no per-pass host read-back). Attributes the
reference uses for its chunk loop and CPU safety net are accepted and recorded:

* ``max_chunk`` / ``mem_fraction`` / ``pinned_transfers``: no effect (the device working set
  is per CTA and does not grow with the batch);
* ``fallback``: only "none" semantics exist -- there is no CPU fallback; a case the frozen
  pivot order does not suit is reported not converged (``last_stats['failed_on_gpu']``);
* ``cpu_handoff``: no stragglers are handed off (finished cases free their slot at once).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from ..solver import GpuSolver, c128


class PolarNewtonSolverCUDA:
    """Device-resident batched polar Newton solver for one grid topology."""

    def __init__(self, Yp, Yj, Yx, pv, pq, reorder: str = "symrcm", backend: str = "lean", slots: int = 32,
                 cases_per_cta: int = 0):
        if backend != "lean":
            raise ValueError("backend must be 'lean' (cuDSS / cusolverRf / cusolverSp backends are not provided)")
        if not 1 <= slots <= 32:
            raise ValueError("slots must be in 1..32")
        self.backend = backend
        self.reorder = reorder
        self.slots = int(slots)
        self.max_chunk = None
        self.mem_fraction = 0.6
        self.precision = "double"
        self.mixed_switch = 1e-3
        # "gb300": float factors until contraction stalls below mixed_switch (default);
        # "reference": the reference's votes (float above mixed_switch, double below it)
        self.vote_rule = "gb300"
        # gb300 rule: a case on float factors iterates until its mismatch is below polish * tol
        # and below vtol / |J^-1| (a bound on the voltage error left)
        self.polish = 1e-3
        self.vtol = 1e-8
        self.line_search = True
        self.fallback = "none"
        self.cpu_handoff = 0
        self.pinned_transfers = True
        # pivot-ratio acceptance bounds relative to the flat-start factorization
        # (nr_polar_solver.py:63-65 _RCOND_RATIO and _rcond_ratio_single)
        self._rcond_ratio = 1e-3
        self._rcond_ratio_single = 1e-3
        self.last_stats: dict = {}
        self._s = GpuSolver(Yp, Yj, Yx, pv, pq, cases_per_cta)
        self.n = self._s.n
        if not np.isfinite(self._s.info["rcond0"]):
            raise RuntimeError(
                "lean LU: the Jacobian has a zero or non-finite diagonal pivot at flat start, so the static pivot "
                "order cannot be used for this grid")

    # ------------------------------------------------------------------ helpers
    def _params(self, max_iter, tol):
        return GpuSolver.params(max_iter, tol, self.line_search, self.precision, self.mixed_switch,
                                pivot_ratio_double=self._rcond_ratio, pivot_ratio_single=self._rcond_ratio_single,
                                vote_rule=self.vote_rule, polish=self.polish, vtol=self.vtol)

    def _record(self, B, r, st=None):
        own = st is None  # a launch of this solver (not of a group): its cases' mismatch is recorded
        st = self._s.stats if st is None else st
        failed = int((~r["converged"]).sum())
        # per-result accuracy: every case's final mismatch and |J^-1| x mismatch, a first-order
        # bound on its voltage's distance from the exact solution (and so from a converged FP64
        # solve); |J^-1| is the topology's estimate from its flat-start factorization
        mis = self._s.last_mismatch(B) if own else None
        jinv = float(self._s.info["jinv_norm"])
        bound = max_mis = None
        if mis is not None:
            r["mismatch"] = mis
            with np.errstate(over="ignore"):  # a failed case's mismatch is DBL_MAX: no bound
                r["error_bound"] = mis * jinv
            ok = np.asarray(r["converged"], bool)
            max_mis = float(mis[ok].max()) if ok.any() else None
            bound = None if max_mis is None else max_mis * jinv
        self.last_stats = {
            "systems": B,
            "chunk": B,
            "chunks": 1,
            "handed_off": 0,
            "failed_on_gpu": failed,
            "fallback": None,
            "single_factorizations": int(st["single_factorizations"]),
            "double_factorizations": int(st["double_factorizations"]),
            "single_rejected": int(st["single_rejected"]),
            "double_rejected": int(st["double_rejected"]),
            "kernel_ms": float(st["kernel_ms"]),
            "grid": int(st["grid"]),
            "cases_per_cta": int(st["cases_per_cta"]),
            # counters of the persistent kernel (beyond the reference's chunk-loop statistics)
            "chord_steps": int(st.get("chord_steps", 0)),
            "first_steps": int(st.get("first_steps", 0)),
            "lazy_jacobians": int(st.get("lazy_jacobians", 0)),
            "jacobian_sweeps": int(st.get("jacobian_sweeps", 0)),
            "jinv_norm": jinv,
            "max_mismatch": max_mis,  # over the converged cases
            "error_bound": bound,     # jinv_norm x max_mismatch
        }
        return r

    @property
    def info(self) -> dict:
        return self._s.info

    # ------------------------------------------------------------------ public API
    def solve_batch(self, Sbus_mat, V0, max_iter: int = 30, tol: float = 1e-8):
        n = self.n
        Sbus_mat = c128(Sbus_mat)
        if Sbus_mat.ndim != 2 or Sbus_mat.shape[0] != n:
            raise ValueError("Sbus must be (n_bus, T)")
        T = Sbus_mat.shape[1]
        V0 = c128(V0)
        if V0.shape not in ((n,), (n, T)):
            raise ValueError("V0 must be (n_bus,) or (n_bus, T)")
        return self._record(T, self._s.solve_batch(Sbus_mat, V0, self._params(max_iter, tol)))

    def solve_timeseries_lanes(self, Sbus_mat, V0, offsets, max_iter: int = 30, tol: float = 1e-8):
        """Hours split into warm-start lanes: hour ``offsets[l] + w`` starts from the converged
        voltage of hour ``offsets[l] + w - 1`` (from V0 for a lane's first hour or after a
        non-converged hour). All lanes run concurrently in one launch."""
        n = self.n
        Sbus_mat = c128(Sbus_mat)
        if Sbus_mat.ndim != 2 or Sbus_mat.shape[0] != n:
            raise ValueError("Sbus must be (n_bus, T)")
        V0 = c128(V0).ravel()
        if V0.shape != (n,):
            raise ValueError("V0 must be (n_bus,)")
        r = self._s.solve_lanes(Sbus_mat, V0, offsets, self._params(max_iter, tol))
        return self._record(Sbus_mat.shape[1], r)

    def _check_contingency_inputs(self, L, Sbus, V0, pin):
        n = self.n
        Sbus = c128(np.asarray(Sbus).ravel())
        V0 = c128(V0)
        pin = np.ascontiguousarray(pin, dtype=np.uint8)
        if Sbus.shape != (n,):
            raise ValueError("Sbus must be (n_bus,)")
        if V0.shape != (n, L) or pin.shape != (n, L):
            raise ValueError("V0/pin must be (n_bus, L)")
        return Sbus, V0, pin

    def solve_batch_contingency_cx(self, Yx, Sbus, V0, pin, max_iter: int = 30, tol: float = 1e-8,
                                   numeric_zero: float = 1e-10, numeric_boost: float = 1e-8):
        Yx = c128(Yx)
        if Yx.ndim != 2 or Yx.shape[0] != self._s.nnz:
            raise ValueError("Yx must be (Ybus nnz, L)")
        L = Yx.shape[1]
        Sbus, V0, pin = self._check_contingency_inputs(L, Sbus, V0, pin)
        return self._record(L, self._s.solve_contingency(Sbus, V0, pin, self._params(max_iter, tol), Yd=Yx))

    def solve_batch_contingency(self, Yx_mag, Yx_ang, Sbus, V0, pin, max_iter: int = 30, tol: float = 1e-8,
                                numeric_zero: float = 1e-10, numeric_boost: float = 1e-8):
        Yx = np.asarray(Yx_mag, dtype=np.float64) * np.exp(1j * np.asarray(Yx_ang, dtype=np.float64))
        return self.solve_batch_contingency_cx(Yx, Sbus, V0, pin, max_iter, tol)

    def solve_batch_contingency_stamp(self, stamp, Sbus, V0, pin, max_iter: int = 30, tol: float = 1e-8,
                                      numeric_zero: float = 1e-10, numeric_boost: float = 1e-8):
        """Per-case Ybus = base values minus column c of the sparse (nnz, L) ``stamp``,
        applied inside the kernel (no per-case Ybus is materialised anywhere)."""
        stamp = sp.csc_matrix(stamp, dtype=np.complex128)
        if stamp.shape[0] != self._s.nnz:
            raise ValueError("stamp must be (Ybus nnz, L)")
        stamp.sum_duplicates()
        L = stamp.shape[1]
        Sbus, V0, pin = self._check_contingency_inputs(L, Sbus, V0, pin)
        st = (stamp.indptr, stamp.indices, stamp.data)
        return self._record(L, self._s.solve_contingency(Sbus, V0, pin, self._params(max_iter, tol), stamps=st))

    def update_Y(self, Yx):
        Yx = c128(Yx)
        if Yx.shape != self._s.Yx.shape:
            raise ValueError("update_Y: nnz mismatch (topology changed; rebuild the solver)")
        if np.array_equal(Yx, self._s.Yx):
            return
        self._s.update_Y(Yx)
        if not np.isfinite(self._s.info["rcond0"]):
            raise RuntimeError("lean LU: the Jacobian has a zero or non-finite diagonal pivot at flat start")

    def free(self):
        """Device memory is released with the solver object."""
        self.last_stats = {}
