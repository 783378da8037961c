"""Autotuner of the Newton kernel's launch: CTA shape and factorization schedule.

The solver picks a CTA shape (threads per CTA, case slots per CTA -- which also fixes the
workers each case's factorization is dealt to) from the batch size by a rule measured on
GB300 (``GpuSolver.shape``), and deals each elimination level's tasks with chains cut at
``chain_cap`` x the level's mean work per worker (``GpuSolver.set_chain_cap``). ``tune``
times every candidate (shape, chain cap) on the caller's real launch and pins the fastest:
the shape for that batch-size class, the chain cap for the solver. Every candidate runs the
same arithmetic per case, so tuning changes only the speed, never a result.
No reference counterpart: the reference's lean LU kernel takes a fixed warps-per-block
``slots`` argument and deals each level to that many lists (p3s/cuda/nr_polar_solver.py:285-300,
p3s/cuda/lean_lu_plan.py:172-190).
"""

from __future__ import annotations

import numpy as np

from .solver import GpuSolver
from .synthetic import lanes

CANDIDATES = ((1024, 1), (1024, 2), (1024, 4), (512, 2), (512, 4), (512, 8), (512, 16), (512, 32), (256, 4),
              (256, 8), (256, 16))


CHAIN_CAPS = (1.0, 0.75, 0.5, 0.35, 0.25, 2.0, 0.0)


def tune(solver: GpuSolver, units: int, run, candidates=CANDIDATES, chain_caps=(1.0,), reps: int = 2):
    """Time `run()` (one launch of `units` work items on `solver`) for every (threads, slots)
    in `candidates` and every chain cap in `chain_caps`; pin the fastest and return it as
    (threads, slots, chain_cap) with the best kernel milliseconds of every candidate."""
    timings = {}
    for cap in chain_caps:
        solver.set_chain_cap(cap)
        for nt, g in candidates:
            solver.set_shape(units, nt, g)
            best = None
            for _ in range(reps + 1):  # the first run builds the shape's schedule and scratch
                run()
                t = solver.stats["kernel_ms"]
                best = t if best is None else min(best, t)
            timings[(nt, g, cap)] = best
    choice = min(timings, key=timings.get)
    solver.set_chain_cap(choice[2])
    solver.set_shape(units, choice[0], choice[1])
    return choice, timings


def _tune(solver: GpuSolver, units: int, run, candidates, reps: int):
    choice, timings = tune(solver, units, run, candidates, (getattr(solver, "chain_cap", 1.0),), reps)
    return choice[:2], {k[:2]: v for k, v in timings.items()}


def tune_lanes(solver: GpuSolver, S, V0, offsets, params, candidates=CANDIDATES, reps: int = 2):
    """Tune the shape for ``solver.solve_lanes(S, V0, offsets, params)``; returns the chosen
    (threads, slots) and the kernel milliseconds of every candidate."""
    S = np.ascontiguousarray(S, dtype=np.complex128)
    K = len(offsets) - 1
    return _tune(solver, K, lambda: solver.solve_lanes(S, V0, offsets, params), candidates, reps)


def tune_batch(solver: GpuSolver, S, V0, params, candidates=CANDIDATES, reps: int = 2):
    """Tune the shape for ``solver.solve_batch(S, V0, params)`` (T = S.shape[1] cases)."""
    S = np.ascontiguousarray(S, dtype=np.complex128)
    T = S.shape[1]
    return _tune(solver, T, lambda: solver.solve_batch(S, V0, params), candidates, reps)


def tune_hours(solver: GpuSolver, S, V0, params, sizes, candidates=CANDIDATES, reps: int = 2):
    """Tune one shape per batch size in `sizes` on the leading hours of S (one lane per hour)."""
    out = {}
    for B in sizes:
        out[B] = tune_lanes(solver, S[:, :B], V0, lanes(B, B), params, candidates, reps)[0]
    return out
