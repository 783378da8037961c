"""The reference's study-level entry points over array grids, on the device.

pandapower is not a dependency of this package, so a "grid" here is any object with the arrays
the reference derives from a net: ``Yp, Yj, Yx`` (CSR Ybus), ``pv, pq, ref`` (bus types),
``Sbus`` (base injections, p.u.), ``V0`` (flat start with the voltage set-points) and, for N-1
studies, the branch table ``f, t, stamp, stamp_pos`` (``p3s_gb300.synthetic.Grid`` is one).

* ``PowerflowObject`` (p3s/PowerflowObject.py:10-32): the plugin interface of the reference's
  Newton loop (``create_J``, ``evaluate_Fx``, ``evaluate_Results``, ``offset``), and
  ``PQPVPowerflowGPU``, its PQ/PV power-flow object (p3s/PQPVPowerflow.py:159-212) with the
  Jacobian and the mismatch computed on the device -- a drop-in for the object the reference's
  ``NewtonPowerflow`` builds (NewtonPowerflow.py:232) in its ``pf_objects``.
* ``calculate_timeseries_cpp`` (p3s/NewtonPowerflowCpp.py:586-676): one start voltage (DC or
  flat), every time step an independent Newton solve of one batched launch; the reference's
  validations, messages and ``LoadflowNotConverged``.
* ``solve_contingencies_cuda`` / ``solve_contingencies_cpp`` (p3s/contingency/solver_cuda.py:
  30-119, solver_cpp.py:64-156): every single-branch outage with islanding and re-slack,
  solved on the device (the CPU-named entry point runs the same device path; ``n_threads`` has
  no effect there).
"""

from __future__ import annotations

from abc import ABC, abstractmethod

import numpy as np
import scipy.sparse as sp

from .cuda.nr_polar_solver import PolarNewtonSolverCUDA
from .solver import GpuSolver, c128


class LoadflowNotConverged(RuntimeError):
    """Raised like pandapower's exception of that name (the reference raises it when a
    time-series batch leaves steps unconverged, NewtonPowerflowCpp.py:671-675)."""


class PowerflowObject(ABC):
    """The reference's plugin interface of one power-flow object in the Newton loop
    (p3s/PowerflowObject.py:10-32): its Jacobian block, its part of the mismatch vector, and
    its voltage update from its slice of the Newton step starting at ``offset``."""

    def __init__(self):
        self._offset: int = 0

    @abstractmethod
    def create_J(self, V):
        pass

    @abstractmethod
    def evaluate_Results(self, dx, voltage):
        pass

    @abstractmethod
    def evaluate_Fx(self, Sbus, V):
        pass

    @property
    def offset(self):
        return self._offset

    @offset.setter
    def offset(self, offset: int):
        self._offset = offset


class PQPVPowerflowGPU(PowerflowObject):
    """PQ/PV buses of one grid (p3s/PQPVPowerflow.py:159-212) with the Jacobian and mismatch
    evaluated by the device kernel of the batched solver: unknowns x = [dVa(pv, pq); dVm(pq)],
    rows [P(pv, pq); Q(pq)]. ``create_J`` returns the CSR triple (Jx, Jp, Jj) the reference's
    object returns (Jp the row pointer, Jj the column indices, sorted within each row)."""

    def __init__(self, YBus, pq, pv, ref):
        super().__init__()
        Y = sp.csr_matrix(YBus, dtype=np.complex128)
        Y.sort_indices()
        self._YBus = Y
        self._pv = np.asarray(pv, dtype=np.int64).ravel()
        self._pq = np.asarray(pq, dtype=np.int64).ravel()
        self._ref = np.asarray(ref, dtype=np.int64).ravel()
        self._pvpq = np.r_[self._pv, self._pq]
        self._n_bus = Y.shape[0]
        self._s = GpuSolver(Y.indptr, Y.indices, Y.data, self._pv, self._pq)

    def _device_J(self, voltage, Sbus=None):
        V = c128(np.asarray(voltage).ravel())
        S = np.zeros(self._n_bus, np.complex128) if Sbus is None else c128(np.asarray(Sbus).ravel())
        return self._s.debug_J(S, V)

    def create_J(self, voltage):
        d = self._device_J(voltage)
        m = d["m"]
        J = sp.csc_matrix((d["Jx"], d["Ji"], d["Jp"]), shape=(m, m)).tocsr()
        J.sort_indices()
        return J.data, J.indptr, J.indices

    def evaluate_Results(self, dx, voltage):
        npq, npv = len(self._pq), len(self._pv)
        Va = np.angle(voltage)
        Vm = np.abs(voltage)
        Va[self._pvpq] += dx[self._offset: self._offset + npv + npq]
        Vm[self._pq] += dx[self._offset + npv + npq: self._offset + npv + 2 * npq]
        return Vm * np.exp(1j * Va)

    def evaluate_Fx(self, Sbus, V):
        return self._device_J(V, Sbus)["F"]


# ---------------------------------------------------------------------------------- studies
def _start_voltage(grid, init: str, solver: GpuSolver, dc_stamps=None, p_shift=None):
    """The shared start of a study: the flat start with the set-points, or with DC angles
    (p3s/timeseries.py:200-247: injections' real part plus the phase-shift injection)."""
    if init == "flat":
        return c128(np.asarray(grid.V0).ravel()).copy()
    if init != "dc":
        raise ValueError(f"init must be 'dc' or 'flat', got {init!r}")
    P = np.asarray(grid.Sbus).real + (0.0 if p_shift is None else np.asarray(p_shift, dtype=np.float64))
    V, _ = solver.dc_start(np.ascontiguousarray(P, dtype=np.float64), grid.V0, dc_stamps=dc_stamps)
    return V


def calculate_timeseries_cpp(grid, sbus_matrix, tolerance: float = 1e-8, max_iterations: int = 30,
                             n_threads: int = 0, init: str = "dc", precision: str = "double", solver=None,
                             dc_stamps=None, p_shift=None):
    """Batched time series (``NewtonPowerflowCpp.calculate_timeseries_cpp``): ``sbus_matrix``
    (n_bus, T) injections per step, one start voltage (``init`` "dc" as the reference, or
    "flat"), every step an independent Newton solve in one launch of the device kernel.
    Returns the converged voltages (n_bus, T); raises ``LoadflowNotConverged`` if any step did
    not converge, ``ValueError`` on the reference's input checks. ``n_threads`` has no effect
    (the reference's OpenMP thread count). ``solver``: a ``PolarNewtonSolverCUDA`` of the grid
    to reuse; ``dc_stamps`` / ``p_shift``: the reference's DC branch model (see ``ybus``)."""
    S = c128(sbus_matrix)
    if S.ndim != 2:
        raise ValueError("Sbus matrix must be (n_bus, T)")
    n_bus, T = S.shape
    if n_bus == 0:
        raise ValueError("Network has no buses")
    if T == 0:
        raise ValueError("Time series has zero time steps")
    if np.any(np.isnan(S)) or np.any(np.isinf(S)):
        raise ValueError("Sbus matrix contains NaN or inf values")
    if solver is None:
        solver = PolarNewtonSolverCUDA(grid.Yp, grid.Yj, grid.Yx, grid.pv, grid.pq)
    if dc_stamps is not None:
        is_slack = np.zeros(n_bus, np.uint8)
        is_slack[np.asarray(grid.ref, dtype=np.int64)] = 1
        solver._s.set_branches(grid.f, grid.t, grid.stamp_pos, grid.stamp, is_slack)
    v_init = _start_voltage(grid, init, solver._s, dc_stamps, p_shift)
    if np.any(np.isnan(v_init)) or np.any(np.isinf(v_init)):
        raise ValueError("DC initial voltage contains NaN or inf values")
    if v_init.shape[0] != n_bus:
        raise ValueError(f"V0 shape mismatch: expected ({n_bus},), got {v_init.shape}")
    solver.precision = precision
    result = solver.solve_batch(S, v_init, max_iter=max_iterations, tol=tolerance)
    if np.any(np.isnan(result["V"])) or np.any(np.isinf(result["V"])):
        raise ValueError("batch solver returned NaN or inf voltages")
    if not bool(np.all(result["converged"])):
        n_bad = int((~np.asarray(result["converged"], bool)).sum())
        raise LoadflowNotConverged(
            f"batch did not converge for {n_bad} of {T} time steps in {max_iterations} iterations.")
    return result["V"]


def solve_contingencies_cuda(grid, reslack_islands: bool = False, tol: float = 1e-8, max_iter: int = 30,
                             init: str = "dc", max_chunk: int | None = None, backend: str = "lean",
                             precision: str = "double", solver=None, dc_stamps=None, p_shift=None):
    """Every N-1 contingency of ``grid`` (the intact grid and each single-branch outage) on the
    device (``solve_contingencies_cuda``): ``init`` picks the shared start ("dc" or "flat"),
    islands are found and re-slacked (``reslack_islands``) inside the solve's launch, unserved
    buses come back NaN. ``max_chunk`` has no effect (one launch holds any batch); ``backend``
    must be "lean". Returns a ``contingency.ContingencyResultTable``."""
    from .contingency import solve_contingencies

    if backend != "lean":
        raise ValueError("backend must be 'lean' (cuDSS / cusolverRf / cusolverSp backends are not provided)")
    if solver is None:
        solver = PolarNewtonSolverCUDA(grid.Yp, grid.Yj, grid.Yx, grid.pv, grid.pq)
    solver.max_chunk = max_chunk
    if dc_stamps is not None:
        is_slack = np.zeros(grid.n, np.uint8)
        is_slack[np.asarray(grid.ref, dtype=np.int64)] = 1
        solver._s.set_branches(grid.f, grid.t, grid.stamp_pos, grid.stamp, is_slack)
        solver._branch_key = None  # the outage path sets its own branch table with priorities
    v_start = _start_voltage(grid, init, solver._s, dc_stamps, p_shift)
    return solve_contingencies(grid, reslack_islands=reslack_islands, tol=tol, max_iter=max_iter,
                               precision=precision, v_start=v_start, solver=solver)


def solve_contingencies_cpp(grid, reslack_islands: bool = False, tol: float = 1e-8, max_iter: int = 30,
                            n_threads: int = 0, init: str = "dc", precision: str = "double", solver=None):
    """``solve_contingencies_cpp`` (p3s/contingency/solver_cpp.py:64-156) under its own name:
    the same cases and semantics, solved by the device path of ``solve_contingencies_cuda``
    (``n_threads`` has no effect)."""
    return solve_contingencies_cuda(grid, reslack_islands=reslack_islands, tol=tol, max_iter=max_iter, init=init,
                                    precision=precision, solver=solver)
