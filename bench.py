"""Benchmark: batched AC power flow solves/s on one GB300 (the 2,000-bus x 8,760-hour series).

One step = one pass of the Newton path over the whole workload: the 2,000-bus grid's
8,760 hourly cases, each hour starting from the converged base case (K = T lanes: the
reference's own time-series semantics), solved to <= 1e-8 p.u. mismatch by ONE launch of the
persistent sm_103a kernel (with its start-table, shared-start and replication prologue kernels).
Beside it (`warm_lanes`): the same hours in K = 730 twelve-hour warm-start lanes, hour h of a
lane starting from hour h-1's converged voltage, with the oracle's replay of the same lanes.

  value : solves/s with inputs resident in HBM (CUDA events around the kernel, solver stream)
  e2e   : solves/s through the public API (p3s_gb300.solver.GpuSolver.solve_lanes_async /
          wait) from pinned host memory, every step copying its inputs in and its results out
          inside the timed region, two steps in flight so one's copies overlap the other's
          kernel (wall clock over the steps); single_call_ms: one call alone
  fp64  : the same for the plain double-precision path (the headline value is the mixed path)
  roofline.phases : the Newton kernel's time split by phase (SM clock counters of one extra
          instrumented launch, shares of the CTA time) with each phase's algorithmic bytes

Beside the headline (rank 0, outside the timed steps): the full N-1 sweep of the same grid
(3,001 cases), the uneven multi-grid batch (256 grids x 16 scenarios in one launch), and the
serving loop (Poisson stream over 32 resident topologies; p50 / p99 latency per rate).

N > 1 (torchrun): every rank solves its own 8,760-hour series (weak scaling, no collective on
the data path); value = all ranks' solves / the slowest rank's time.
`--impl reference` times the CPU oracle (the restatement of the reference's nr_klu solver,
all host cores) on the same workload.
"""

from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "parallel-pandapower-solver_gb300"), ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "solves/s on 1 GB300, mixed vs FP64 at ≤1e-8 pu mismatch; p50/p99 latency"
N_BUS, HOURS = 2000, 8760


def shard(B: int, rank: int, world: int):
    """Contiguous [lo, hi) share of B cases for `rank` of `world` (every case exactly once)."""
    base, extra = divmod(B, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


# ----------------------------------------------------------------------------- distributed
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- workload
def workload(rank: int = 0, hours: int = HOURS):
    from p3s_gb300.synthetic import grid_2000, timeseries_injections

    g = grid_2000(0)
    S = timeseries_injections(g, hours, seed=1 + rank)
    return g, S


def shared_start(g):
    """The lanes' shared start voltage: the converged base case (solved once by the CPU
    oracle, outside any timed region) -- the role the reference's DC start plays for its
    time series (p3s/timeseries.py:200-244)."""
    from oracle import cpu

    r = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).solve_batch(g.Sbus[:, None], g.V0)
    assert r["converged"][0]
    return np.ascontiguousarray(r["V"][:, 0])


# autotune candidates of the headline launch: the rule's shape and its neighbours
TUNE_SHAPES = ((512, 32), (512, 16), (1024, 32), (1024, 16))
# ... of the uneven multi-grid launch: (threads per CTA, 0 = the rule; variable buses x case
# slots a CTA takes per job, the group rule's 16,384 and its neighbours)
MG_PACKING = ((0, 16384), (0, 8192), (0, 32768), (512, 4096), (1024, 16384))
# ... and of the N-1 sweep's launch (3,001 cases; 0 = the group rule: 512 x 16)
N1_SHAPES = ((0, 0), (512, 8), (512, 32), (1024, 8), (1024, 16), (256, 4), (256, 8))


def n_lanes(T, cases_per_cta=32, threads_per_cta=512, nsm=None):
    """Warm-start lanes: one per case slot of the launch (SMs x resident CTAs x slots), at most
    one per hour. K = T starts every hour from the shared start (the reference's semantics)."""
    if nsm is None:
        import torch

        nsm = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 152
    return min(T, nsm * (1024 // threads_per_cta) * cases_per_cta)


def algorithmic_bytes(info: dict, g, mixed: bool):
    """Bytes a case-iteration must move (the hot path's per-unit traffic model), split into the
    part every iteration moves -- eval (V state, S, Jacobian write, residual), solve (read LU
    and residual, write step), step (read step, rewrite the state) -- and the refactorization
    (read A, write LU), which a chord step leaves out. Index arrays are shared by the batch
    and excluded. b = 8 (double path) or 4 (float Jacobian/LU in the mixed path)."""
    n = g.n
    m = len(g.pv) + 2 * len(g.pq)  # scalar unknowns
    from p3s_gb300.topology import jacobian_pattern

    nnzJ = len(jacobian_pattern(g.Yp, g.Yj, g.pv, g.pq)[1])
    nnzLU = 4 * info["n_blocks"]
    b = 4 if mixed else 8
    per_iteration = (3 * n * 8 + 2 * n * 8 + b * nnzJ + 8 * m) + (b * nnzLU + 16 * m) + (8 * m + 6 * n * 8)
    per_factorization = b * nnzJ + b * nnzLU
    return per_iteration, per_factorization


def phase_bytes(info: dict, g, mixed: bool, iterations: int, factorizations: int) -> dict:
    """The traffic model split by the Newton kernel's phases for one launch: the evaluation;
    the factorization fused with the forward substitution (the refactorization term per
    factorization, plus half of the substitutions' term per case-iteration); the backward
    substitution (the other half); the voltage update. Refill / load and the decision move no
    modelled bytes."""
    n = g.n
    m = len(g.pv) + 2 * len(g.pq)
    from p3s_gb300.topology import jacobian_pattern

    nnzJ = len(jacobian_pattern(g.Yp, g.Yj, g.pv, g.pq)[1])
    nnzLU = 4 * info["n_blocks"]
    b = 4 if mixed else 8
    half_solve = b * nnzLU / 2 + 8 * m
    return {"eval": iterations * (3 * n * 8 + 2 * n * 8 + b * nnzJ + 8 * m),
            "factor_forward": factorizations * (b * nnzJ + b * nnzLU) + iterations * half_solve,
            "backward": iterations * half_solve, "step": iterations * (8 * m + 6 * n * 8), "load": 0.0,
            "decide": 0.0}


def phase_table(cycles: dict, kernel_ms: float, bytes_: dict, peak: float) -> dict:
    """Per phase: its share of the kernel's CTA time (SM clock counters), that share of the
    kernel time, its algorithmic bytes and the bandwidth they make over that time."""
    total = float(sum(cycles.values())) or 1.0
    out = {}
    for k, c in cycles.items():
        share = c / total
        ms = share * kernel_ms
        gb = bytes_.get(k, 0.0) / 1e9
        row = {"share": round(share, 4), "ms": round(ms, 3), "algorithmic_GB": round(gb, 3)}
        if gb > 0 and ms > 0:
            row["achieved_GBps"] = round(gb / (ms * 1e-3), 1)
            row["frac"] = round(gb / (ms * 1e-3) / peak, 4)
        out[k] = row
    return out


def headline_config(g, T: int, K: int) -> dict:
    """The timed workload, the same dict in the GPU line and the reference line."""
    return {
        "workload": f"2,000-bus grid x {T} hourly cases, K={K} warm-start lanes (hour h of a lane starts from "
                    f"hour h-1's converged voltage, a lane's first hour from the converged base case; K = {T}: "
                    f"every hour starts from the converged base case, the reference's time-series semantics)",
        "n_bus": g.n, "n_branch": g.n_branch, "n_pv": len(g.pv), "n_pq": len(g.pq), "hours": T, "lanes": K,
        "tol_pu": 1e-8, "max_iter": 30,
        "injection_scale": round(float(g.loading), 6),
        "start": "the converged base case, solved once outside the timed region",
        "l2": "inputs larger than L2 (S is 280 MB per step; L2 is 129 MB)",
    }


def algorithmic_bytes_per_iteration(info: dict, g, mixed: bool) -> float:
    """The model's bytes of a case-iteration that refactors."""
    it, fac = algorithmic_bytes(info, g, mixed)
    return it + fac


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv",
                                          "-lms", "100", "-f", self.path], stdout=subprocess.DEVNULL,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(", ") for r in open(self.path).read().strip().splitlines()[1:]]
        os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1].split()[0]))
                mx.append(float(r[2].split()[0]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def load_traffic():
    """DRAM bytes per case-iteration of the Newton kernel from the committed ncu summary."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", "newton_kernel_traffic.json")))
    except Exception:
        return {}


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, local):
    import torch

    from p3s_gb300 import _lib
    from p3s_gb300.solver import GpuSolver, pinned_empty
    from p3s_gb300.synthetic import lanes

    torch.cuda.set_device(local)
    _lib.require_device()
    g, S = workload(rank, args.hours)
    V0 = shared_start(g)
    T = S.shape[1]
    solver = GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    info = solver.info
    K = args.lanes or n_lanes(T, info["cases_per_cta"], info["threads_per_cta"])
    off = lanes(T, K).astype(np.int64)
    dev = torch.device("cuda", local)
    dS = torch.from_numpy(S.view(np.float64).copy()).to(dev)
    dV0 = torch.from_numpy(V0.view(np.float64).copy()).to(dev)
    doff = torch.from_numpy(off).to(dev)
    dV = torch.empty(2 * g.n * T, dtype=torch.float64, device=dev)
    dit = torch.empty(T, dtype=torch.int32, device=dev)
    dcv = torch.empty(T, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()

    def dev_step(p):
        solver.solve_lanes_device(dS.data_ptr(), dV0.data_ptr(), doff.data_ptr(), T, len(off) - 1, p, dV.data_ptr(),
                                  dit.data_ptr(), dcv.data_ptr())
        return solver.stats

    # the launch shape (threads, case slots per CTA) and the factorization schedule's chain cap
    # of this workload, per precision, measured before the timed steps (autotune): every
    # candidate solves the same cases to the same bits, only the time differs
    tuned = {}

    def use(prec):
        if prec in tuned:
            t = tuned[prec]
            solver.set_chain_cap(t["chain_cap"])
            solver.set_shape(K, t["threads_per_cta"], t["cases_per_cta"])

    out = {}
    for prec in ("mixed", "double"):
        p = GpuSolver.params(precision=prec, mixed_switch=args.mixed_switch)
        if not args.no_tune:
            from p3s_gb300 import autotune

            choice, timings = autotune.tune(solver, K, lambda: dev_step(p), candidates=TUNE_SHAPES,
                                            chain_caps=autotune.CHAIN_CAPS, reps=1)
            tuned[prec] = {"threads_per_cta": choice[0], "cases_per_cta": choice[1], "chain_cap": choice[2],
                           "kernel_ms": {f"{k[0]}x{k[1]} cap {k[2]:g}": round(v, 3) for k, v in timings.items()}}
        use(prec)
        for _ in range(args.warmup):
            dev_step(p)
        barrier(world)
        torch.cuda.synchronize()
        ms, its, stats = [], [], None
        clocks = Clocks(local)
        with clocks:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                stats = dev_step(p)
                ms.append(stats["kernel_ms"])
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        barrier(world)
        it = dit.cpu().numpy()
        cv = dcv.cpu().numpy().astype(bool)
        out[prec] = dict(ms=float(np.mean(ms)), wall_ms=wall * 1e3 / args.steps, it=it, cv=cv, stats=stats,
                         clocks=clocks.summary())

    # the Newton kernel's time by phase: one instrumented launch per precision, outside the timed
    # steps (SM clock counters at the phase barriers, summed over the CTAs)
    for prec in ("mixed", "double"):
        use(prec)
        dev_step(GpuSolver.params(precision=prec, mixed_switch=args.mixed_switch, phase_timers=True))
        out[prec]["phase_cycles"] = solver.stats["phase_cycles"]

    # the same hours in K = 730 twelve-hour warm-start lanes (hour h from hour h-1's converged
    # voltage): both precisions timed like the headline, the oracle's replay of the same lanes
    # on the host cores beside them
    K_warm = min(730, T)
    off_w = lanes(T, K_warm).astype(np.int64)
    doff_w = torch.from_numpy(off_w).to(dev)
    warm = {"lanes": K_warm}
    for prec in ("mixed", "double"):
        p = GpuSolver.params(precision=prec, mixed_switch=args.mixed_switch)

        def warm_step():
            solver.solve_lanes_device(dS.data_ptr(), dV0.data_ptr(), doff_w.data_ptr(), T, K_warm, p, dV.data_ptr(),
                                      dit.data_ptr(), dcv.data_ptr())
            return solver.stats["kernel_ms"]

        for _ in range(args.warmup):
            warm_step()
        ms = [warm_step() for _ in range(max(3, args.steps // 2))]
        it = dit.cpu().numpy()
        warm["fp64" if prec == "double" else prec] = {
            "value": round(world * T / (np.mean(ms) * 1e-3), 1), "unit": "solves/s",
            "ms_per_step": round(float(np.mean(ms)), 3), "iterations_mean": float(it.mean()),
            "converged": bool(dcv.cpu().numpy().all())}
    if rank == 0:
        best = min(cpu_solve(g, S, K_warm, V0)[0] for _ in range(3))
        warm["cpu_baseline"] = {"value": round(T / best, 1), "unit": "solves/s", "cores": cpu_cores(), "kind": "port",
                                "sample": f"all {T} hours in the same {K_warm} lanes (the oracle's lane replay), "
                                          f"best of 3, oracle/liboracle.so (OpenMP, {cpu_cores()} threads)"}

    # accuracy of the mixed result against the oracle's mismatch on a few hours (the mixed
    # launch configuration from here on: the end-to-end steps below are mixed)
    use("mixed")
    p = GpuSolver.params(precision="mixed", mixed_switch=args.mixed_switch)
    dev_step(p)
    V = dV.cpu().numpy().view(np.complex128).reshape(g.n, T)
    from oracle import cpu

    osv = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    hrs = np.linspace(0, T - 1, 8).astype(int)
    worst_mis = max(float(np.abs(osv.debug_J_at(S[:, h], V[:, h])["F"]).max()) for h in hrs)
    # voltages of the mixed path against the double path at the same tolerance (the oracle's
    # iterations; it stops anywhere below tol) and against a converged double solve (tol 1e-12)
    Vd = {}
    for tol in (1e-8, 1e-12):
        dev_step(GpuSolver.params(precision="double", tol=tol))
        Vd[tol] = dV.cpu().numpy().view(np.complex128).reshape(g.n, T)

    def dv(a, b):
        return {"max_dVm": float(np.abs(np.abs(a) - np.abs(b)).max()),
                "max_dVa_rad": float(np.abs(np.angle(a * np.conj(b))).max())}

    accuracy = {"mixed_vs_fp64_path": dv(V, Vd[1e-8]), "mixed_vs_converged_fp64": dv(V, Vd[1e-12]),
                "fp64_path_vs_converged_fp64": dv(Vd[1e-8], Vd[1e-12])}

    # end to end through the public API from pinned host buffers: consecutive steps in two
    # slots, so one step's copies overlap the other's kernel (every step still copies its
    # inputs in and its results out inside the timed region); wall clock over all steps
    bufs = []
    for _ in range(2):
        Sh = pinned_empty(S.shape, np.complex128)
        Sh[...] = S
        bufs.append((Sh, pinned_empty((g.n, T), np.complex128), pinned_empty((T,), np.int32),
                     pinned_empty((T,), np.uint8)))
    V0h = pinned_empty(V0.shape, np.complex128)
    V0h[...] = V0
    p = GpuSolver.params(precision="mixed", mixed_switch=args.mixed_switch)

    def pipelined(steps):
        for k in range(steps):
            slot = k % 2
            if k >= 2:
                solver.wait(slot)
            Sh, Vh, ith, cvh = bufs[slot]
            solver.solve_lanes_async(slot, Sh, V0h, off, p, out=(Vh, ith, cvh))
        for k in range(max(0, steps - 2), steps):
            solver.wait(k % 2)

    pipelined(args.warmup)
    barrier(world)
    t0 = time.perf_counter()
    pipelined(args.steps)
    e2e_wall = (time.perf_counter() - t0) * 1e3 / args.steps
    barrier(world)
    # the same call alone (no overlap with a neighbour): device time from first copy in to last out
    single = []
    for _ in range(3):
        Sh, Vh, ith, cvh = bufs[0]
        solver.solve_lanes(Sh, V0h, off, p, out=(Vh, ith, cvh))
        single.append(solver.stats["call_ms"])
    assert np.array_equal(bufs[0][1], bufs[1][1]) and np.array_equal(bufs[0][2], bufs[1][2])
    h2d = S.nbytes + V0.nbytes + off.nbytes
    d2h = bufs[0][1].nbytes + bufs[0][2].nbytes + bufs[0][3].nbytes

    res = dict(out=out, e2e_ms=e2e_wall, e2e_single_ms=float(np.min(single)), h2d=h2d, d2h=d2h, info=info,
               K=len(off) - 1, T=T, worst_mis=worst_mis, g=g, accuracy=accuracy, polish=p.polish, vtol=p.vtol,
               warm=warm, tuned=tuned)
    return res


def run_n1(args):
    """The full N-1 sweep of the same grid (base case + every single-branch outage, 3,001
    cases): device islanding with re-slack, then one stamp-patched solve, through the public
    driver (host arrays in and out). Reported beside the time series, not as the headline."""
    from p3s_gb300 import contingency
    from p3s_gb300.cuda.nr_polar_solver import PolarNewtonSolverCUDA
    from p3s_gb300.synthetic import grid_2000

    g = grid_2000(0)
    solver = PolarNewtonSolverCUDA(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    out = {"cases": g.n_branch + 1}
    for prec in ("mixed", "double"):
        cap_ms, shape_ms = {}, {}
        shape = (0, 0)
        if not args.no_tune:
            # the launch's CTA shape (threads, case slots per CTA) and the factorization schedule's
            # chain cap, measured (autotune): the same results for every candidate, only the time
            # differs
            from p3s_gb300 import autotune

            def timed(nt, cpc):
                t = []
                for _ in range(2):
                    contingency.solve_contingencies(g, reslack_islands=True, precision=prec, solver=solver,
                                                    return_islands=False, cases_per_cta=cpc, threads_per_cta=nt)
                    t.append(solver.last_stats["kernel_ms"])
                return min(t)

            solver._s.set_chain_cap(1.0)
            for nt, cpc in N1_SHAPES:
                shape_ms[(nt, cpc)] = timed(nt, cpc)
            shape = min(shape_ms, key=shape_ms.get)
            for cap in autotune.CHAIN_CAPS:
                solver._s.set_chain_cap(cap)
                cap_ms[cap] = timed(*shape)
            solver._s.set_chain_cap(min(cap_ms, key=cap_ms.get))

        def solve():
            return contingency.solve_contingencies(g, reslack_islands=True, precision=prec, solver=solver,
                                                   return_islands=False, cases_per_cta=shape[1],
                                                   threads_per_cta=shape[0])

        for _ in range(args.warmup):
            r = solve()
        wall, kern = [], []
        for _ in range(max(1, args.steps // 2)):
            t0 = time.perf_counter()
            r = solve()
            wall.append(time.perf_counter() - t0)
            kern.append(solver.last_stats["kernel_ms"])
        L = g.n_branch + 1
        out["fp64" if prec == "double" else prec] = {
            "value": round(L / (np.mean(kern) * 1e-3), 1), "unit": "solves/s", "kernel_ms": round(float(np.mean(kern)), 3),
            "e2e_solves_per_s": round(L / np.mean(wall), 1), "e2e_ms": round(float(np.mean(wall)) * 1e3, 1),
            "iterations_mean": float(r.iterations.mean()), "converged": int(r.converged.sum()),
            "islanded_cases": int((r.served.sum(axis=0) < g.n).sum()),
            "chain_cap": solver._s.chain_cap,
            "chain_cap_ms": {f"{k:g}": round(v, 3) for k, v in cap_ms.items()} or None,
            "shape": list(shape) if shape != (0, 0) else "group rule",
            "shape_ms": {f"{k[0]}x{k[1]}": round(v, 3) for k, v in shape_ms.items()} or None,
        }
    return out


def run_multigrid(args):
    """256 synthetic grids with bus counts log-uniform in [30, 20,000] (1.5 n branches, 10 % PV
    buses), 16 load scenarios each (base loads x U(0.8, 1.2)): ONE persistent launch over all
    of them (a group), against the same grids solved one launch per grid."""
    from p3s_gb300.group import GpuGroup, GroupJob
    from p3s_gb300.solver import GpuSolver
    from p3s_gb300.synthetic import multigrid_batch

    grids, scen = multigrid_batch()
    solvers = [GpuSolver(g.Yp, g.Yj, g.Yx, g.pv, g.pq) for g in grids]
    grp = GpuGroup()
    jobs = [GroupJob(s, S, g.V0) for s, S, g in zip(solvers, scen, grids)]
    cases = sum(S.shape[1] for S in scen)
    out = {"grids": len(grids), "cases": cases, "bus_range": [min(g.n for g in grids), max(g.n for g in grids)]}
    for prec in ("mixed", "double"):
        p = GpuSolver.params(precision=prec)
        tuned = None
        if not args.no_tune:
            # the launch's packing (threads per CTA; variable buses x case slots a CTA takes per
            # job, i.e. cases per CTA by grid size) and the factorization schedule's chain cap,
            # measured (autotune): the same results for every candidate, only the time differs
            from p3s_gb300 import autotune

            def timed():
                t = []
                for _ in range(2):
                    grp.solve(jobs, p)
                    t.append(grp.stats["kernel_ms"])
                return min(t)

            for s in solvers:
                s.set_chain_cap(1.0)
            packing = {}
            for nt, budget in MG_PACKING:
                grp.set_shape(nt, budget)
                packing[(nt, budget)] = timed()
            best = min(packing, key=packing.get)
            grp.set_shape(*best)
            caps = {}
            for cap in autotune.CHAIN_CAPS:
                for s in solvers:
                    s.set_chain_cap(cap)
                caps[cap] = timed()
            cap = min(caps, key=caps.get)
            for s in solvers:
                s.set_chain_cap(cap)
            tuned = {"threads_per_cta": best[0] or "rule", "slot_budget": best[1], "chain_cap": cap,
                     "packing_ms": {f"{k[0] or 'rule'}x{k[1]}": round(v, 3) for k, v in packing.items()},
                     "chain_cap_ms": {f"{k:g}": round(v, 3) for k, v in caps.items()}}
        for _ in range(args.warmup):
            res = grp.solve(jobs, p)
        kern, call = [], []
        for _ in range(max(1, args.steps // 2)):
            res = grp.solve(jobs, p)
            kern.append(grp.stats["kernel_ms"])
            call.append(grp.stats["call_ms"])
        per_grid = 0.0
        for s, S, g in zip(solvers, scen, grids):
            s.solve_batch(S, g.V0, p)
            per_grid += s.stats["kernel_ms"]
        its = np.concatenate([r["iterations"] for r in res])
        cv = np.concatenate([r["converged"] for r in res])
        out["fp64" if prec == "double" else prec] = {
            "value": round(cases / (np.mean(kern) * 1e-3), 1), "unit": "solves/s", "kernel_ms": round(float(np.mean(kern)), 3),
            "e2e_solves_per_s": round(cases / (np.mean(call) * 1e-3), 1),
            "one_launch_per_grid_kernel_ms": round(per_grid, 2),
            "iterations_mean": float(its.mean()), "converged": int(cv.sum()),
            "threads_per_cta": grp.stats["threads_per_cta"], "grid_ctas": grp.stats["grid"],
            "autotune": tuned,
        }
    return out


def run_serving(args):
    """Poisson request stream over 32 resident topologies of 100..50,000 buses (70 % single
    solves, 25 % 96-step chunks, 5 % 200-outage N-1 sweeps), served with continuous batching;
    the rate is raised until p99 latency exceeds 50 ms. Latency = completion - arrival (wall
    clock, host arrays in and out). Primary (``mixed`` / ``fp64``): the stream server -- one
    running launch that takes each request as it arrives (slot-level admission); beside it
    (``contexts``): the launch-context server, whose requests wait for a free launch."""
    from p3s_gb300.serving import Server, StreamServer, Topology, latency_summary, poisson_stream
    from p3s_gb300.stream import GpuStream
    from p3s_gb300.synthetic import make_grid

    rng = np.random.default_rng(5)
    sizes = np.sort(np.exp(rng.uniform(np.log(100), np.log(50000), 32)).astype(int))
    topos = [Topology(make_grid(int(n), seed=500 + i, max_drop_pu=0.05)) for i, n in enumerate(sizes)]
    out = {"topologies": len(topos), "bus_range": [int(sizes[0]), int(sizes[-1])], "stream_s": args.serve_seconds}
    from p3s_gb300.group import GpuGroup

    def sweep_rates(srv):
        sweep = []
        for rate in (25, 50, 100, 200, 280, 400, 560, 800, 1130, 1600):
            reqs = poisson_stream(topos, rate=float(rate), duration=args.serve_seconds, seed=rate)
            gc.collect()
            gc.disable()
            try:
                resp = srv.run(reqs, keep_results=False)
            finally:
                gc.enable()
            st = latency_summary(resp)
            w = max(resp, key=lambda r: r.latency)
            q = reqs[w.rid]
            st["slowest"] = {"kind": q.kind, "n_bus": int(topos[q.topo].n), "cases": int(len(w.iterations)),
                             "wait_ms": round((w.start - w.arrival) * 1e3, 2),
                             "run_ms": round((w.done - w.start) * 1e3, 2), "arrival_s": round(w.arrival, 3)}
            sweep.append({"rate_per_s": rate, **{k: (round(v, 3) if isinstance(v, float) else v) for k, v in st.items()}})
            if st["p99_ms"] > 50.0:
                break
        ok = [x for x in sweep if x["p99_ms"] <= 50.0]
        best = ok[-1] if ok else None
        return {"max_rate_p99_le_50ms": best["rate_per_s"] if best else None,
                "solves_per_s": best["solves_per_s"] if best else None,
                "p50_ms": best["p50_ms"] if best else None, "p99_ms": best["p99_ms"] if best else None,
                "sweep": sweep}

    # the stream server: one running launch per stream, requests admitted as they arrive
    backend = GpuStream(capacity=32768, arena_bytes=16 << 30, result_bytes=8 << 30)
    for prec in ("mixed", "double"):
        srv = StreamServer(topos, precision=prec, backend=backend)
        srv.run(poisson_stream(topos, rate=200.0, duration=0.5, seed=1), keep_results=False)  # warm-up
        row = {"server": "stream (slot-level admission into one running launch)"}
        if prec == "mixed":
            # per topology and request kind, the precision that finishes a request sooner in the
            # running launch (measured alone, both ways): large grids' latency-bound requests
            # may run on double factors
            chosen = srv.tune()
            row["precision"] = ("mixed launch; per topology and request kind the precision measured faster "
                                "at warm-up (StreamServer.tune)")
            row["double_by_kind"] = {k: sum(1 for (t, kk), p in chosen.items() if kk == k and p == "double")
                                     for k in ("single", "chunk", "n1")}
        out["fp64" if prec == "double" else prec] = {**row, **sweep_rates(srv)}
    del backend
    out["contexts"] = {}
    groups = [GpuGroup() for _ in range(4)]  # both context servers run on the same 4 launch contexts
    for prec in ("mixed", "double"):
        srv = Server(topos, precision=prec, groups=groups, pinned_results=True)
        srv.warmup(cases=96, n1_outages=200)  # the stream's largest chunk and N-1 sweep
        sweep = []
        # rates in steps of sqrt(2) from 200 req/s, where the 50 ms bound starts to bind
        for rate in (25, 50, 100, 200, 280, 400, 560, 800, 1130, 1600):
            reqs = poisson_stream(topos, rate=float(rate), duration=args.serve_seconds, seed=rate)
            # the host's garbage collector paused during the stream (a collection over the
            # bench's large arrays would stall the serving loop for 100s of ms)
            gc.collect()
            gc.disable()
            try:
                resp = srv.run(reqs, keep_results=False)  # each result dropped once on the host
            finally:
                gc.enable()
            s = latency_summary(resp)
            # the slowest request: what it was, how long it waited for a launch and ran in one
            w = max(resp, key=lambda r: r.latency)
            q = reqs[w.rid]
            s["slowest"] = {"kind": q.kind, "n_bus": int(topos[q.topo].n), "cases": int(len(w.iterations)),
                            "wait_ms": round((w.start - w.arrival) * 1e3, 2), "run_ms": round((w.done - w.start) * 1e3, 2),
                            "arrival_s": round(w.arrival, 3),
                            "launch_requests": int(sum(1 for r in resp if r.launch == w.launch))}
            sweep.append({"rate_per_s": rate, **{k: (round(v, 3) if isinstance(v, float) else v) for k, v in s.items()}})
            if s["p99_ms"] > 50.0:
                break
        ok = [x for x in sweep if x["p99_ms"] <= 50.0]
        best = ok[-1] if ok else None
        out["contexts"]["fp64" if prec == "double" else prec] = {
            "server": "4 launch contexts (a request waits for a free launch)",
            "max_rate_p99_le_50ms": best["rate_per_s"] if best else None,
            "solves_per_s": best["solves_per_s"] if best else None,
            "p50_ms": best["p50_ms"] if best else None, "p99_ms": best["p99_ms"] if best else None,
            "sweep": sweep}
    return out


def solver_chain_cap(res, prec):
    t = res.get("tuned") or {}
    return t[prec]["chain_cap"] if prec in t else 1.0


def gpu_line(args, res, rank, world):
    out = res["out"]
    T = res["T"]
    mixed, dbl = out["mixed"], out["double"]
    ms_mixed = reduce_max(mixed["ms"], world)
    ms_dbl = reduce_max(dbl["ms"], world)
    e2e_ms = reduce_max(res["e2e_ms"], world)
    if rank != 0:
        return None
    g = res["g"]
    info = res["info"]
    value = world * T / (ms_mixed * 1e-3)
    peaks = load_peaks()
    hbm = peaks.get("hbm_gbs")
    its_mixed = int(mixed["it"].sum())
    B = algorithmic_bytes_per_iteration(info, g, True)
    B_it, B_fac = algorithmic_bytes(info, g, True)
    n_fac = int(mixed["stats"]["single_factorizations"] + mixed["stats"]["double_factorizations"])
    launch_bytes = B_it * its_mixed + B_fac * n_fac  # chord steps leave the refactorization out
    achieved = launch_bytes / (mixed["ms"] * 1e-3) / 1e9
    traffic = load_traffic()
    tr = traffic.get("mixed_bytes_per_case_iteration")
    roof = {
        "bound": "hbm",
        "achieved": round(achieved, 1),
        "peak": hbm if hbm else 6800.0,
        "unit": "GB/s",
        "frac": round(achieved / (hbm if hbm else 6800.0), 4),
        "traffic": None if tr is None else float(tr) * its_mixed,
        "traffic_source": None if tr is None else "ncu DRAM bytes per case-iteration of one launch of the "
                                                  "2,000-bus x 2,432-hour case (profiles/newton_kernel_traffic.json) "
                                                  "x this launch's case-iterations",
        "peak_source": "measured" if hbm else "fallback",
        "kernel": "newton_kernel",
        "algorithmic_bytes_per_case_iteration": B,
        "algorithmic_bytes_per_launch": launch_bytes,
        "case_iterations_per_launch": its_mixed,
        "factorizations_per_launch": n_fac,
        "chord_steps_per_launch": int(mixed["stats"].get("chord_steps", 0)),
        "first_steps_per_launch": int(mixed["stats"].get("first_steps", 0)),
    }
    peak = hbm if hbm else 6800.0
    roof["phases"] = phase_table(mixed["phase_cycles"], mixed["ms"],
                                 phase_bytes(info, g, True, its_mixed, n_fac), peak)
    roof["phases_source"] = ("SM clock counters at the Newton kernel's phase barriers, summed over its CTAs, of one "
                             "instrumented launch (gbpf_params.phase_timers); ms = the phase's share of the CTA time x "
                             "the timed kernel time; bytes from the per-case-iteration traffic model")
    its_dbl = int(dbl["it"].sum())
    n_fac_dbl = int(dbl["stats"]["single_factorizations"] + dbl["stats"]["double_factorizations"])
    # fp64 pipe roofline of the double path (GB300: ~1.2 TFLOP/s)
    fp64 = {
        "value": round(world * T / (ms_dbl * 1e-3), 1),
        "ms_per_step": round(ms_dbl, 3),
        "iterations_mean": float(dbl["it"].mean()),
        "converged": bool(dbl["cv"].all()),
        "achieved_GBps": round(algorithmic_bytes_per_iteration(info, g, False) * int(dbl["it"].sum())
                               / (dbl["ms"] * 1e-3) / 1e9, 1),
        "clocks": dbl["clocks"],
        "phases": phase_table(dbl["phase_cycles"], dbl["ms"], phase_bytes(info, g, False, its_dbl, n_fac_dbl), peak),
    }
    cb = cpu_baseline(res["g"], args, res["K"])
    line = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_mixed, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 Jacobian/LU + f64 mismatch/update",
        "data": "synthetic (seeded 2,000-bus grid and 8,760-hour load/generation series)",
        "config": headline_config(g, T, res["K"]),
        "run": {
            "precision": "mixed", "mixed_switch": args.mixed_switch, "shared_start": True,
            "cases_per_cta": mixed["stats"]["cases_per_cta"], "threads_per_cta": mixed["stats"]["threads_per_cta"],
            "grid_ctas": mixed["stats"]["grid"], "chain_cap": solver_chain_cap(res, "mixed"),
            "iterations_mean": float(mixed["it"].mean()), "converged": bool(mixed["cv"].all()),
            "max_mismatch_pu_sampled": res["worst_mis"],
            "polish": res["polish"], "vtol": res["vtol"], "jinv_norm_est": info["jinv_norm"],
            "single_factorizations": int(mixed["stats"]["single_factorizations"]),
            "double_factorizations": int(mixed["stats"]["double_factorizations"]),
            "lazy_jacobians": int(mixed["stats"].get("lazy_jacobians", 0)),
            "jacobian_sweeps": int(mixed["stats"].get("jacobian_sweeps", 0)),
        },
        "fp64": fp64,
        "warm_lanes": res["warm"],
        "autotune": res["tuned"] or None,
        "accuracy": res["accuracy"],
        "n1_sweep": res.get("n1"),
        "multigrid": res.get("multigrid"),
        "serving": res.get("serving"),
        "roofline": roof,
        "cpu_baseline": cb,
        "e2e": {"value": round(world * T / (e2e_ms * 1e-3), 1), "unit": "solves/s",
                "h2d_bytes_per_step": int(res["h2d"]), "d2h_bytes_per_step": int(res["d2h"]),
                "ms_per_step": round(e2e_ms, 3),
                "timing": "wall clock over the timed steps, two steps in flight (gbpf_solve_lanes_async)",
                "single_call_ms": round(res["e2e_single_ms"], 3)},
        "clocks": mixed["clocks"],
        # per step: the start-state table, the shared start and its replication, the Newton kernel
        "gpu_launches": 4 * args.steps,
        "wall_ms_per_step": round(mixed["wall_ms"], 3),
    }
    return line


# ----------------------------------------------------------------------------- CPU arms
def cpu_solve(g, S, K, V0):
    from oracle import cpu
    from p3s_gb300.synthetic import lanes

    s = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    off = lanes(S.shape[1], K)
    t0 = time.perf_counter()
    r = cpu.solve_lanes(s, S, V0, off)
    return time.perf_counter() - t0, r


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline(g, args, lanes_used):
    """The oracle (restated nr_klu, OpenMP over all usable cores) on a bounded sample of the
    same workload: the first `cpu_hours` hours in the same lane structure, best of 3."""
    from oracle.build import build_oracle

    build_oracle()
    hours = min(args.cpu_hours, HOURS)
    _, S = workload(0, hours)
    K = max(1, round(hours * lanes_used / HOURS))
    V0 = shared_start(g)
    best = min(cpu_solve(g, S, K, V0)[0] for _ in range(3))
    return {"value": round(hours / best, 1), "unit": "solves/s", "cores": cpu_cores(), "kind": "port",
            "sample": f"first {hours} of the {HOURS} hours, {K} warm-start lanes, best of 3, oracle/liboracle.so "
                      f"(OpenMP, {cpu_cores()} threads)"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle.build import build_oracle
    from p3s_gb300.synthetic import grid_2000

    build_oracle()
    g = grid_2000(0)
    hours = min(args.cpu_hours, HOURS)
    _, S = workload(0, hours)
    K = max(1, round(hours * (args.lanes or n_lanes(HOURS, nsm=152)) / HOURS))
    V0 = shared_start(g)
    for _ in range(args.warmup):
        cpu_solve(g, S, K, V0)
    times = [cpu_solve(g, S, K, V0)[0] for _ in range(args.steps)]
    ms = float(np.mean(times)) * 1e3
    value = hours / (ms * 1e-3)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded 2,000-bus grid and hourly load/generation series)",
        "config": headline_config(g, hours, K),
        "cpu_baseline": {"value": round(value, 1), "unit": "solves/s", "cores": cpu_cores(), "kind": "port",
                         "sample": f"{hours} hours per step on all host cores (oracle/liboracle.so, a restatement "
                                   f"of the reference's nr_klu; the reference's own build needs its checkout)"},
        "e2e": {"value": round(value, 1), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--hours", type=int, default=HOURS)
    ap.add_argument("--lanes", type=int, default=0, help="warm-start lanes (0: one per case slot, at most T)")
    ap.add_argument("--mixed-switch", type=float, default=1e-3)
    ap.add_argument("--cpu-hours", type=int, default=HOURS)
    ap.add_argument("--no-n1", action="store_true", help="skip the N-1 sweep block")
    ap.add_argument("--no-multigrid", action="store_true", help="skip the uneven multi-grid block")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving block")
    ap.add_argument("--no-tune", action="store_true", help="keep the solver's shape rule (no autotune)")
    ap.add_argument("--serve-seconds", type=float, default=4.0, help="length of each serving stream")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":  # rank 0 alone times the CPU reference; other ranks exit at once
        rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, rank, world)
        return
    rank, world, local = dist_init()
    res = run_gpu(args, rank, world, local)
    if rank == 0 and not args.no_n1:
        res["n1"] = run_n1(args)
    if rank == 0 and not args.no_multigrid:
        res["multigrid"] = run_multigrid(args)
    if rank == 0 and not args.no_serving:
        res["serving"] = run_serving(args)
    line = gpu_line(args, res, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
