"""CTA-shape autotuner: time candidate shapes on a caller's batch and pin the fastest.

The solver picks a CTA shape (threads per CTA, case slots per CTA) from the batch size by a
rule measured on GB300 (``GpuSolver.shape``). For a grid or batch size the rule was not
measured on, ``tune_lanes`` / ``tune_batch`` time every candidate shape on the real inputs
and pin the fastest for that batch-size class (``GpuSolver.set_shape``). Every shape runs
the same arithmetic per case, so tuning changes only the speed, never a result.
No reference counterpart: the reference's lean LU kernel takes a fixed warps-per-block
``slots`` argument (p3s/cuda/nr_polar_solver.py:285-300).
"""

from __future__ import annotations

import numpy as np

from .solver import GpuSolver
from .synthetic import lanes

CANDIDATES = ((1024, 1), (1024, 2), (1024, 4), (512, 2), (512, 4), (512, 8), (512, 16), (512, 32), (256, 4),
              (256, 8), (256, 16))


def _tune(solver: GpuSolver, units: int, run, candidates, reps: int):
    timings = {}
    for nt, g in candidates:
        solver.set_shape(units, nt, g)
        best = None
        for _ in range(reps + 1):  # the first run builds the shape's schedule and scratch
            run()
            t = solver.stats["kernel_ms"]
            best = t if best is None else min(best, t)
        timings[(nt, g)] = best
    choice = min(timings, key=timings.get)
    solver.set_shape(units, *choice)
    return choice, timings


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
