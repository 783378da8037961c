"""N-1 contingency batch on the device: outage stamps, islanding, re-slack, solve.

Counterpart of the reference's ``p3s/contingency/case_generator.py`` (stamp map, served
masks, island references) and ``solver_cuda.py`` / ``solver_cpp.py`` (V0 / pin assembly,
batched solve, NaN at unserved buses), for grids given as arrays (the reference reads
pandapower nets, which this package does not depend on):

* each outage group subtracts its branches' exact 2x2 stamps at their 4 CSR positions
  (case_generator.py:270-317, 505-524) -- handed to the kernel as sparse per-case stamps,
  no per-case Ybus is materialised;
* islands: connected components of the live branch graph minus the group, on the device
  (``gbpf_islands``), numbered like scipy's connected_components;
* references: an island with a slack stays served; with ``reslack_islands`` an island
  without one is re-slacked to its generator of highest priority (default: the largest
  scheduled active power, ties to the lowest bus index -- the reference ranks by
  short-circuit impedance, which array grids do not carry); other islands are unserved;
* V0 / pin (solver_cpp.py:121-134): re-slack buses pinned at |v0| + 0j, unserved buses at
  1 + 0j; unserved voltages are returned as NaN.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

from . import _lib
from .cuda.nr_polar_solver import PolarNewtonSolverCUDA


@dataclass
class ContingencyBatch:
    Yp: np.ndarray
    Yj: np.ndarray
    Yx_base: np.ndarray
    n_bus: int
    groups: list  # branch indices of every case (an empty list: the intact grid)
    pv: np.ndarray
    pq: np.ndarray
    ref: np.ndarray
    f: np.ndarray
    t: np.ndarray
    live: np.ndarray  # (nbr,) branch couples its two ends (Y_ft or Y_tf nonzero)
    stamp: sp.csc_matrix  # (nnz, L) values subtracted from the base Ybus

    @property
    def Yx_matrix(self) -> np.ndarray:
        """Dense (nnz, L) per-case values (for the dense API and the oracle)."""
        return np.asarray(self.Yx_base[:, None] - self.stamp.toarray())

    @property
    def outages(self):
        ptr = np.zeros(len(self.groups) + 1, dtype=np.int32)
        ptr[1:] = np.cumsum([len(g) for g in self.groups])
        idx = np.concatenate([np.asarray(g, dtype=np.int32) for g in self.groups]) if ptr[-1] else np.zeros(
            0, np.int32)
        return ptr, idx.astype(np.int32)


@dataclass
class ContingencyResultTable:
    groups: list
    V: np.ndarray  # (n, L) complex, NaN at unserved buses
    served: np.ndarray  # (n, L) bool
    converged: np.ndarray  # (L,) bool
    iterations: np.ndarray  # (L,) int
    labels: np.ndarray = None  # (n, L) int32 island of every bus
    ref_bus: np.ndarray = None  # (n, L) int32 reference bus of every bus's island, -1 unserved

    @property
    def vm(self) -> np.ndarray:
        return np.abs(self.V)

    @property
    def va(self) -> np.ndarray:
        return np.degrees(np.angle(self.V))


def build_batch(grid, groups=None, include_base: bool = True) -> ContingencyBatch:
    """Cases from a synthetic ``Grid``: by default the intact grid plus every single-branch
    outage (``groups`` overrides: a list of branch-index lists)."""
    nbr = grid.n_branch
    if groups is None:
        groups = ([[]] if include_base else []) + [[b] for b in range(nbr)]
    rows, cols, vals = [], [], []
    for c, g in enumerate(groups):
        for b in g:
            rows.append(grid.stamp_pos[b])
            cols.append(np.full(4, c))
            vals.append(grid.stamp[b])
    nnz = grid.nnz
    L = len(groups)
    if rows:
        stamp = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                              shape=(nnz, L)).tocsc()
    else:
        stamp = sp.csc_matrix((nnz, L), dtype=np.complex128)
    stamp.sum_duplicates()
    stamp.sort_indices()
    live = (grid.stamp[:, 1] != 0) | (grid.stamp[:, 2] != 0)
    return ContingencyBatch(grid.Yp, grid.Yj, grid.Yx, grid.n, [list(map(int, g)) for g in groups], grid.pv, grid.pq,
                            grid.ref, grid.f, grid.t, live, stamp)


def islands(batch: ContingencyBatch, reslack_islands: bool, gen_prio=None):
    """(labels (n, L) int32, served (n, L) bool, ref_bus (n, L) int32, n_islands (L,)) on the device."""
    L_ = _lib.require_device()
    n = batch.n_bus
    Lc = len(batch.groups)
    f = np.ascontiguousarray(batch.f, dtype=np.int32)
    t = np.ascontiguousarray(batch.t, dtype=np.int32)
    live = np.ascontiguousarray(batch.live, dtype=np.uint8)
    ptr, idx = batch.outages
    is_slack = np.zeros(n, dtype=np.uint8)
    is_slack[np.asarray(batch.ref, dtype=np.int64)] = 1
    prio = np.zeros(n) if gen_prio is None else np.ascontiguousarray(gen_prio, dtype=np.float64)
    labels = np.empty((n, Lc), dtype=np.int32)
    served = np.empty((n, Lc), dtype=np.uint8)
    ref_bus = np.empty((n, Lc), dtype=np.int32)
    nis = np.empty(Lc, dtype=np.int32)
    rc = L_.gbpf_islands(n, len(f), _lib.i32(f), _lib.i32(t), _lib.u8(live), Lc, _lib.i32(ptr), _lib.i32(idx),
                         _lib.u8(is_slack), _lib.d(prio), int(bool(reslack_islands)), _lib.i32(labels),
                         _lib.u8(served), _lib.i32(ref_bus), _lib.i32(nis))
    _lib.check(rc, "gbpf_islands")
    return labels, served.astype(bool), ref_bus, nis


def start_and_pins(batch: ContingencyBatch, v_start, served, ref_bus):
    """Per-case V0 and pin mask (solver_cpp.py:119-134): re-slack buses at |v0| + 0j,
    unserved buses at 1 + 0j, both pinned."""
    n, Lc = served.shape
    v_start = np.asarray(v_start, dtype=np.complex128)
    V0 = np.repeat(v_start[:, None], Lc, axis=1)
    pin = np.zeros((n, Lc), dtype=np.uint8)
    is_slack = np.zeros(n, dtype=bool)
    is_slack[np.asarray(batch.ref, dtype=np.int64)] = True
    # re-slack references: buses that are the reference of their island but not a slack
    bus = np.arange(n)[:, None]
    is_ref = (ref_bus == bus) & ~is_slack[:, None]
    V0[is_ref] = np.abs(np.broadcast_to(v_start[:, None], V0.shape)[is_ref]) + 0j
    pin[is_ref] = 1
    V0[~served] = 1.0 + 0.0j
    pin[~served] = 1
    return np.ascontiguousarray(V0), np.ascontiguousarray(pin)


def outage_lists(groups):
    """(ptr (L+1,), idx) int32 outage lists of case groups (branch index lists)."""
    ptr = np.zeros(len(groups) + 1, dtype=np.int32)
    ptr[1:] = np.cumsum([len(g) for g in groups])
    idx = np.fromiter(itertools.chain.from_iterable(groups), dtype=np.int32, count=int(ptr[-1]))
    return ptr, idx


def single_outage_lists(n_branch: int):
    """outage_lists of the base case and every single-branch outage ([[], [0], ..., [m-1]]),
    made directly."""
    ptr = np.arange(-1, n_branch + 1, dtype=np.int32)
    ptr[0] = 0
    return ptr, np.arange(n_branch, dtype=np.int32)


def solve_contingencies(grid, reslack_islands: bool = False, tol: float = 1e-8, max_iter: int = 30,
                        precision: str = "double", groups=None, gen_prio=None, v_start=None, solver=None,
                        return_islands: bool = True, cases_per_cta: int = 0, threads_per_cta: int = 0):
    """Solve every N-1 case of ``grid`` on the device (``solve_contingencies_cuda`` semantics,
    solver_cuda.py:30-119, with ``init="flat"``).

    The grid's branch table stays resident with the solver; every case is an outage list, so
    islanding, the re-slack start and the outage-patched Ybus are all made on the device in the
    solve's launch (no per-case arrays cross the bus but the results). Unserved buses come back
    as NaN; ``served`` is the launch's own islanding mask. ``return_islands`` adds the island
    labels and reference buses (one more islanding call). ``cases_per_cta`` /
    ``threads_per_cta``: the launch's CTA shape (0: the group rule), e.g. from a tuner."""
    from .group import GpuGroup, GroupJob

    n = grid.n
    if groups is None:
        groups = [[]] + [[b] for b in range(grid.n_branch)]
        outages = single_outage_lists(grid.n_branch)
    else:
        groups = [list(map(int, g)) for g in groups]
        outages = outage_lists(groups)
    if len(groups) == 0:
        e = np.empty((n, 0))
        return ContingencyResultTable([], e.astype(np.complex128), e.astype(bool), np.empty(0, bool),
                                      np.empty(0, int))
    if gen_prio is None:
        gen_prio = np.zeros(n)
        gen_prio[grid.pv] = np.maximum(grid.p_gen[grid.pv], np.finfo(float).tiny)
    gen_prio = np.ascontiguousarray(gen_prio, dtype=np.float64)
    if v_start is None:
        v_start = grid.V0
    if solver is None:
        solver = PolarNewtonSolverCUDA(grid.Yp, grid.Yj, grid.Yx, grid.pv, grid.pq)
    gs = solver._s
    key = (id(grid), gen_prio.tobytes())
    if getattr(solver, "_branch_key", None) != key:
        is_slack = np.zeros(n, dtype=np.uint8)
        is_slack[np.asarray(grid.ref, dtype=np.int64)] = 1
        gs.set_branches(grid.f, grid.t, grid.stamp_pos, grid.stamp, is_slack, gen_prio)
        solver._branch_key = key
    if getattr(solver, "_group", None) is None:
        solver._group = GpuGroup()
    solver._group.set_shape(threads_per_cta, 0)
    solver.precision = precision
    job = GroupJob(gs, np.asarray(grid.Sbus), np.asarray(v_start), n_cases=len(groups), outages=outages,
                   reslack=reslack_islands, cases_per_cta=cases_per_cta)
    res = solver._group.solve([job], solver._params(max_iter, tol), pinned_out=True)[0]
    solver._record(len(groups), res, solver._group.stats)
    V = res["V"]
    served = res["served"]
    labels = ref_bus = None
    if return_islands:
        batch = build_batch(grid, groups)
        labels, _, ref_bus, _ = islands(batch, reslack_islands, gen_prio)
    return ContingencyResultTable(groups, V, served, np.asarray(res["converged"], bool),
                                  np.asarray(res["iterations"], int), labels, ref_bus)
