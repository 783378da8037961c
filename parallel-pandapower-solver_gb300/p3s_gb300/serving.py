"""Serving loop: continuous batching of power-flow requests over resident topologies.

A ``Server`` keeps every registered topology resident on the device -- Ybus, plan and
schedules (``GpuSolver``), its warm-start voltage (the converged base case) and its N-1
data -- and serves a stream of requests:

* ``single``: one operating point (n,) of injections;
* ``chunk``: a time-series chunk (n, T), every step starting from the warm-start voltage;
* ``n1``: an N-1 sweep over a list of branch outages (islands, re-slack, stamp-patched Ybus).

Requests are admitted as they arrive. Whenever one of the server's launch contexts
(``GpuGroup``: its own stream and scratch) is free, every admitted request joins ONE
persistent-kernel launch (largest job first), within the launch's case limit and the
device-memory budget; requests that arrive while launches run wait at most until the next
context frees, and the launches of different contexts overlap on the device, on one topology
or on several (a topology's plan and schedules are read-only while it serves). Some contexts
take small requests only (at most ``small_work`` bus-cases), so a burst of large requests
holding the other contexts does not queue the small ones behind it. A time-series
chunk or an N-1 sweep is a job of its own, solved straight from the caller's array into its
own result array; the single solves of one topology share a job. Every case runs the same
arithmetic alone and in any mix, so a request's result does not depend on what it was
batched with.

No reference counterpart: the reference solves one call at a time
(p3s/cuda/nr_polar_solver.py:466-596, p3s/contingency/solver_cuda.py:30-119); its N-1
semantics (islands, re-slack, V0 / pin) are those of ``contingency``.
"""

from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from .group import GpuGroup, GroupJob
from .solver import GpuSolver, c128, pool_keep_at_least, pooled_empty


@dataclass
class Request:
    rid: int
    topo: int                 # index of a registered topology
    kind: str                 # "single" | "chunk" | "n1"
    arrival: float            # seconds from the start of the stream
    S: np.ndarray             # (n,) or (n, T) injections (n1: the base-case injections)
    outages: np.ndarray | None = None  # n1: branch indices, one outage case each


@dataclass
class Response:
    rid: int
    V: np.ndarray             # (n, T) complex; n1: NaN at unserved buses
    iterations: np.ndarray
    converged: np.ndarray
    arrival: float
    start: float              # launch start (seconds from the start of the stream)
    done: float
    launch: int               # launch sequence number
    served: np.ndarray | None = None

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def _slot_bytes(n: int, nv: int, nblk: int, mixed: bool) -> int:
    """Device bytes of one case slot (the kernel's per-slot scratch, gbpf::scratch_offsets):
    double factors and inverse diagonals, residual and step, two state buffers, (e, f), 1/Vm in
    double and float, pins; mixed: two float factor buffers and the float step."""
    nf = nblk + nv
    b = nf * 32 + nv * 32 + n * (32 + 32 + 16 + 8 + 4 + 1)
    if mixed:
        b += 2 * nf * 16 + nv * 8
    return b


class Topology:
    """A resident grid: solver, warm-start voltage and N-1 data."""

    def __init__(self, grid, name: str = ""):
        self.grid = grid
        self.name = name or f"{grid.n}-bus"
        self.solver = GpuSolver(grid.Yp, grid.Yj, grid.Yx, grid.pv, grid.pq)
        info = self.solver.info
        self.n = grid.n
        self.nv = info["n_var_bus"]
        self.nblk = info["n_blocks"]
        base = self.solver.solve_batch(grid.Sbus[:, None], grid.V0, GpuSolver.params(precision="double"))
        if not base["converged"][0]:
            raise RuntimeError(f"{self.name}: the base case does not converge")
        self.V_warm = np.ascontiguousarray(base["V"][:, 0])
        self.f = np.ascontiguousarray(grid.f, dtype=np.int32)
        self.is_slack = np.zeros(self.n, dtype=np.uint8)
        self.is_slack[np.asarray(grid.ref, dtype=np.int64)] = 1
        self.prio = np.zeros(self.n)
        self.prio[grid.pv] = np.maximum(grid.p_gen[grid.pv], np.finfo(float).tiny)
        # the branch table stays resident: N-1 cases are islanded and patched on the device
        self.solver.set_branches(grid.f, grid.t, grid.stamp_pos, grid.stamp, self.is_slack, self.prio)

    def slot_bytes(self, mixed: bool) -> int:
        return _slot_bytes(self.n, self.nv, self.nblk, mixed)

    def n1_job(self, outages: np.ndarray, S_base: np.ndarray) -> GroupJob:
        """Single-branch outage cases from the warm start: the launch islands them, re-slacks
        islands (each starting rotated to its new reference) and patches the Ybus on the device."""
        L = len(outages)
        ptr = np.arange(L + 1, dtype=np.int32)
        idx = np.ascontiguousarray(outages, dtype=np.int32)
        return GroupJob(self.solver, c128(S_base).ravel(), self.V_warm, n_cases=L, outages=(ptr, idx), reslack=True)


@dataclass
class _Launch:
    seq: int
    requests: list
    jobs: list
    served: dict = field(default_factory=dict)  # rids of N-1 requests (served = not NaN)
    start: float = 0.0


class Server:
    """Continuous batching over resident topologies (see the module docstring).

    precision: "mixed" or "double"; contexts: launches that may overlap on the device, of
    which small_contexts take only requests of at most small_work bus-cases (buses x cases);
    max_cases: cases per launch; hbm_budget: bytes of case-slot scratch all contexts may hold;
    slot_budget: variable buses x case slots a CTA holds per job (smaller than bulk launches':
    a request's cases spread over more CTAs, which keeps its latency down); groups: launch
    contexts to serve on (e.g. another server's, whose grown buffers are then reused instead of
    released and allocated again), else `contexts` new ones; pinned_results: results of 1 MB or
    more land in pooled page-locked host memory (no page faults in the copy; a block returns to
    the pool when its response is dropped), and `warmup` fills the pool for the largest requests.
    """

    def __init__(self, topologies: list[Topology], precision: str = "mixed", contexts: int = 2,
                 max_cases: int = 8192, hbm_budget: float = 64e9, tol: float = 1e-8, max_iter: int = 30,
                 slot_budget: int = 8192, small_contexts: int = 0, small_work: int = 1 << 18,
                 groups: list[GpuGroup] | None = None, pinned_results: bool = False, **solver_params):
        self.topos = topologies
        # no shared-start prologue ahead of a request's launch: latency first
        solver_params.setdefault("shared_start", False)
        self.params = GpuSolver.params(max_iter=max_iter, tol=tol, precision=precision, **solver_params)
        self.mixed = precision == "mixed"
        self.groups = list(groups) if groups else [GpuGroup() for _ in range(max(1, contexts))]
        # the last small_contexts contexts serve small requests only (never all of them)
        self.small = set(range(len(self.groups) - min(max(0, small_contexts), len(self.groups) - 1),
                               len(self.groups)))
        self.small_work = small_work
        self.pinned_results = pinned_results
        self.slot_budget = slot_budget
        for grp in self.groups:  # fewer case slots per CTA than bulk launches: more CTAs per request
            grp.set_shape(0, slot_budget)
        self.max_cases = max_cases
        self.hbm_budget = hbm_budget
        self._cv = threading.Condition()

    def warmup(self, cases: int = 64, n1_outages: int = 64):
        """Build every topology's schedules and grow every context's scratch and staging
        buffers before serving, so that no launch allocates device memory (an allocation or
        release synchronises the device and would stall the launches in flight). cases: the
        largest time-series chunk expected; n1_outages: the largest N-1 sweep expected (each
        context runs one launch with that many cases on every topology, which sizes its buffers
        for any mix of smaller requests)."""
        big = max(self.topos, key=lambda tp: tp.nblk)
        for tp in self.topos:  # every shape a request's launch may take (its group's slot rule)
            g = 1
            while g * 2 <= 32 and g * 2 * max(1, tp.nv) <= self.slot_budget:
                g *= 2
            tp.solver.prepare_shapes(g)
        for grp in self.groups:
            jobs = [GroupJob(tp.solver, tp.grid.Sbus, tp.V_warm, n_cases=1) for tp in self.topos]
            jobs.append(GroupJob(big.solver, big.grid.Sbus, big.V_warm, n_cases=max(cases, 1)))
            jobs += [GroupJob(tp.solver, tp.grid.Sbus, tp.V_warm, n_cases=cases) for tp in self.topos]
            grp.solve(jobs, self.params)
            grp.solve([tp.n1_job(np.arange(min(n1_outages, len(tp.f)), dtype=np.int32), tp.grid.Sbus)
                       for tp in self.topos], self.params)
        if self.pinned_results:  # page-locked blocks for every context's largest results
            held = []
            for tp in self.topos:
                for _ in self.groups:
                    for shape, dt in (((tp.n, cases), np.complex128), ((tp.n, n1_outages), np.complex128),
                                      ((tp.n, n1_outages), np.uint8)):
                        if shape[0] * shape[1] * np.dtype(dt).itemsize >= 1 << 20:
                            held.append(pooled_empty(shape, dt))
            pool_keep_at_least(2 * sum(a.nbytes for a in held))
            del held  # the blocks go back to the pool

    # ------------------------------------------------------------------ batching
    def _cases(self, r: Request) -> int:
        if r.kind == "n1":
            return len(r.outages)
        return 1 if r.S.ndim == 1 else r.S.shape[1]

    def _footprint(self, r: Request) -> float:
        return self._cases(r) * self.topos[r.topo].slot_bytes(self.mixed)

    def _is_small(self, r: Request) -> bool:
        return self._cases(r) * self.topos[r.topo].n <= self.small_work

    def _form(self, pending: deque, budget_left: float, small_only: bool = False):
        """Take pending requests, oldest first, within the launch's case and memory limits
        (the oldest is taken even when it alone exceeds them); small_only: small requests only."""
        take, cases, mem = [], 0, 0.0
        keep = deque()
        while pending:
            r = pending.popleft()
            c, fp = self._cases(r), self._footprint(r)
            if (small_only and not self._is_small(r)) or (take and (cases + c > self.max_cases or mem + fp > budget_left)):
                keep.append(r)
                continue
            take.append(r)
            cases += c
            mem += fp
        pending.extend(keep)
        return take, mem

    def _jobs(self, reqs: list):
        """Jobs of one launch: the single solves of a topology together (columns of one
        (n, k) array), every chunk and every N-1 sweep alone -- a job of its own reads the
        request's array in place and its result array is the response's, so a large request
        is not copied on the host. layout[j]: (request, first column, end column) per job."""
        singles = {}
        jobs, layout, served = [], [], {}
        for r in reqs:
            tp = self.topos[r.topo]
            if r.kind == "single":
                singles.setdefault(r.topo, []).append(r)
            elif r.kind == "n1":
                jobs.append(tp.n1_job(r.outages, r.S))
                layout.append([(r, 0, len(r.outages))])
                served[r.rid] = True
            else:
                S = r.S if r.S.ndim == 2 else r.S[:, None]
                jobs.append(GroupJob(tp.solver, S, tp.V_warm))
                layout.append([(r, 0, S.shape[1])])
        for k, rs in singles.items():
            tp = self.topos[k]
            S = rs[0].S[:, None] if len(rs) == 1 else np.stack([r.S for r in rs], axis=1)
            jobs.append(GroupJob(tp.solver, S, tp.V_warm))
            layout.append([(r, c, c + 1) for c, r in enumerate(rs)])
        return jobs, layout, served

    # ------------------------------------------------------------------ serving
    def run(self, requests: list[Request], realtime: bool = True, keep_results: bool = True) -> list[Response]:
        """Serve a request stream. realtime: each request is admitted at its arrival time
        (wall clock from the call); otherwise all are admitted at once. keep_results False:
        each voltage result is dropped once it is on the host (its response keeps the
        iterations, flags and times), as a server does once it has sent it."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending: deque = deque()
        responses: dict[int, Response] = {}
        free = list(range(len(self.groups)))
        mem_in_use = [0.0]
        inflight = [0]
        errors: list = []
        seq = [0]
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def worker(gi: int, launch: _Launch, mem: float, layout):
            try:
                res = self.groups[gi].solve(launch.jobs, self.params, pinned_out=self.pinned_results)
                done = now()
                out = []
                for job_res, spans in zip(res, layout):
                    whole = len(spans) == 1  # the job's result arrays are the response's
                    for r, a, b in spans:
                        V = job_res["V"] if whole else job_res["V"][:, a:b].copy()
                        it = job_res["iterations"] if whole else job_res["iterations"][a:b].copy()
                        cv = job_res["converged"] if whole else job_res["converged"][a:b].copy()
                        sv = job_res["served"] if r.rid in launch.served else None  # an N-1 job is one request
                        if not keep_results:
                            V = sv = None
                            it, cv = it.copy(), cv.copy()
                        out.append(Response(r.rid, V, it, cv, r.arrival, launch.start, done, launch.seq, sv))
            except Exception as e:  # reported to the caller after the stream
                out = []
                errors.append(e)
            with self._cv:
                for resp in out:
                    responses[resp.rid] = resp
                free.append(gi)
                mem_in_use[0] -= mem
                inflight[0] -= 1
                self._cv.notify_all()

        i = 0
        with self._cv:
            while i < len(reqs) or pending or inflight[0]:
                tnow = now()
                while i < len(reqs) and (not realtime or reqs[i].arrival <= tnow):
                    pending.append(reqs[i])
                    i += 1
                if errors:
                    break
                if pending and free:
                    # a general context if one is free, else a small-request one
                    gi = next((g for g in free if g not in self.small), free[0])
                    take, mem = self._form(pending, self.hbm_budget - mem_in_use[0], gi in self.small)
                    if take:
                        free.remove(gi)
                        jobs, layout, served = self._jobs(take)
                        launch = _Launch(seq[0], take, jobs, served, now())
                        seq[0] += 1
                        mem_in_use[0] += mem
                        inflight[0] += 1
                        threading.Thread(target=worker, args=(gi, launch, mem, layout), daemon=True).start()
                        continue
                wait = None
                if i < len(reqs) and realtime:
                    wait = max(0.0, reqs[i].arrival - now())
                if wait is None and not inflight[0] and not pending:
                    continue
                self._cv.wait(timeout=wait if wait is not None else 0.05)
        if errors:
            raise errors[0]
        return [responses[r.rid] for r in requests]


def latency_summary(responses: list[Response], elapsed: float | None = None) -> dict:
    """p50 / p99 latency (ms) and solves/s of a served stream."""
    lat = np.array([r.latency for r in responses]) * 1e3
    cases = int(sum(len(r.iterations) for r in responses))
    span = elapsed if elapsed is not None else (max(r.done for r in responses) - min(r.arrival for r in responses))
    conv = float(np.mean(np.concatenate([r.converged for r in responses])))
    return {"requests": len(responses), "cases": cases, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
            "solves_per_s": cases / span if span > 0 else float("nan"), "converged_fraction": conv}


def poisson_stream(topos: list[Topology], rate: float, duration: float, seed: int = 0, chunk: int = 96,
                   n1_outages: int = 200, mix=(0.70, 0.25, 0.05)) -> list[Request]:
    """Seeded Poisson request stream: single solves, time-series chunks and N-1 sweeps in the
    proportions `mix`, each on a topology drawn uniformly; loads scaled U(0.8, 1.2)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        k = int(rng.integers(len(topos)))
        tp = topos[k]
        g = tp.grid
        u = rng.random()
        kind = "single" if u < mix[0] else ("chunk" if u < mix[0] + mix[1] else "n1")
        if kind == "single":
            S = g.Sbus.copy()
            S[g.pq] *= rng.uniform(0.8, 1.2, len(g.pq))
            out.append(Request(len(out), k, kind, t, S))
        elif kind == "chunk":
            S = np.repeat(g.Sbus[:, None], chunk, axis=1)
            S[g.pq, :] *= rng.uniform(0.8, 1.2, (len(g.pq), chunk))
            out.append(Request(len(out), k, kind, t, np.ascontiguousarray(S)))
        else:
            nb = len(g.f)
            L = min(n1_outages, nb)
            outs = np.sort(rng.choice(nb, L, replace=False)).astype(np.int32)
            out.append(Request(len(out), k, kind, t, g.Sbus.copy(), outs))
    return out


class StreamServer:
    """Slot-level admission: ONE persistent launch (``stream.GpuStream``) serves the stream.
    Every request becomes a job of its own the moment it arrives -- its inputs are staged and
    its descriptor appended to the running launch -- and the kernel's CTAs take it as soon as
    they run out of cases of earlier jobs; its results land in page-locked host memory and its
    flag is polled here. Requests therefore never wait for another launch to finish. Staging and
    result memory are reused as jobs finish (a request waits only while they are all held by
    running jobs); when a launch's ring of job slots is used up, the server stops it (it finishes
    every job it took), starts a new one and goes on, and a launch that returned at its idle limit
    is replaced the same way, its unstarted jobs submitted again.

    Same request and response types as ``Server``; every case runs the same arithmetic as in
    any other launch, so each result equals the one it gets alone (bit for bit). ``backend``:
    the launch object (a ``GpuStream`` by default; tests may pass a stand-in).

    A mixed-precision server can run some jobs on double factors: ``tune`` measures, per
    topology and request kind, which precision finishes a request sooner in the running launch
    and keeps that choice (``precision_of``). On large grids a request's cases run one per CTA,
    latency-bound, where float factors save little per iteration and the float path's extra
    polish iterations cost more than they save."""

    def __init__(self, topologies: list[Topology], precision: str = "mixed", tol: float = 1e-8, max_iter: int = 30,
                 capacity: int = 8192, arena_bytes: int = 8 << 30, result_bytes: int = 4 << 30,
                 idle_seconds: float = 10.0, backend=None, threads: int = 1024, **solver_params):
        self.topos = topologies
        solver_params.setdefault("shared_start", False)
        self.params = GpuSolver.params(max_iter=max_iter, tol=tol, precision=precision, **solver_params)
        self.idle_seconds = idle_seconds
        if backend is None:
            from .stream import GpuStream

            backend = GpuStream(capacity=capacity, arena_bytes=arena_bytes, result_bytes=result_bytes, threads=threads)
        self.backend = backend
        self.launches = 0
        self.precision_of: dict = {}  # (topology, kind) -> "double" / "mixed" (tune); else the launch's

    def _start(self):
        self.backend.start([tp.solver for tp in self.topos], self.params, self.idle_seconds)
        self.launches += 1

    def _submit(self, r: Request):
        tp = self.topos[r.topo]
        prec = self.precision_of.get((r.topo, r.kind))
        if r.kind == "n1":
            L = len(r.outages)
            outages = (np.arange(L + 1, dtype=np.int32), np.ascontiguousarray(r.outages, dtype=np.int32))
            return self.backend.submit(tp.solver, r.S, tp.V_warm, outages=outages, reslack=True, precision=prec)
        return self.backend.submit(tp.solver, r.S, tp.V_warm, precision=prec)

    def _time_copies(self, r: Request, copies: int) -> float:
        """Seconds from submitting `copies` copies of `r` together to the running launch until
        the last one's flag is set (a launch that is full, or has left at its idle limit, is
        renewed first). Several copies weigh a request's GPU work as well as its latency: a
        large grid's request runs one case per CTA, and its copies compete for the SMs."""
        for _ in range(3):
            if self.backend.full() or not self.backend.alive():
                self.backend.stop()
                self._start()
            t0 = time.perf_counter()
            subs = [self._submit(r) for _ in range(copies)]
            if any(sub is None for sub in subs):  # staging held by earlier jobs: renew the launch
                self.backend.stop()
                self._start()
                continue
            qs = [sub[0] for sub in subs]
            while not all(self.backend.flags()[q] for q in qs) and self.backend.alive():
                time.sleep(2e-5)
            if all(self.backend.flags()[q] for q in qs):
                dt = time.perf_counter() - t0
                for q in qs:
                    self.backend.done(q)
                    self.backend.release(q)
                return dt
            self.backend.stop()  # the launch left before starting the jobs: renew and submit again
            self._start()
        raise RuntimeError("tune: a request did not complete in three launches")

    def tune(self, chunk: int = 96, n1_outages: int = 200, repeats: int = 3, seed: int = 0,
             copies: int = 3) -> dict:
        """For a mixed-precision server: per topology and request kind (single solve, chunk of
        `chunk` steps, sweep of `n1_outages` outages), submit `copies` requests of that kind
        together to a running launch in each precision, `repeats` times, and keep the precision
        whose median completion time is shorter. Returns {(topology, kind): precision}."""
        if self.params.precision != 1:
            return {}
        rng = np.random.default_rng(seed)
        reqs = []
        for k, tp in enumerate(self.topos):
            g = tp.grid
            S1 = g.Sbus.copy()
            S1[g.pq] *= rng.uniform(0.8, 1.2, len(g.pq))
            Sc = np.repeat(g.Sbus[:, None], chunk, axis=1)
            Sc[g.pq, :] *= rng.uniform(0.8, 1.2, (len(g.pq), chunk))
            nb = len(g.f)
            outs = np.sort(rng.choice(nb, min(n1_outages, nb), replace=False)).astype(np.int32)
            reqs += [Request(0, k, "single", 0.0, S1), Request(0, k, "chunk", 0.0, np.ascontiguousarray(Sc)),
                     Request(0, k, "n1", 0.0, g.Sbus.copy(), outs)]
        self.precision_of = {}
        times: dict = {}
        self._start()
        try:
            for r in reqs:
                for prec in ("mixed", "double"):
                    self.precision_of[(r.topo, r.kind)] = prec
                    for _ in range(repeats):
                        times.setdefault((r.topo, r.kind, prec), []).append(self._time_copies(r, copies))
        finally:
            self.backend.stop()
        self.precision_of = {
            (r.topo, r.kind): min(("mixed", "double"), key=lambda p: float(np.median(times[(r.topo, r.kind, p)])))
            for r in reqs}
        return dict(self.precision_of)

    def run(self, requests: list[Request], realtime: bool = True, keep_results: bool = True) -> list[Response]:
        """Serve a request stream (``Server.run``'s semantics). A response's ``start`` is the
        moment its job was handed to the running launch; ``launch`` counts the launches."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        responses: dict[int, Response] = {}
        pending: deque = deque()
        outstanding: dict[int, tuple] = {}
        # the server is up -- its launch running -- before the stream's clock starts (a launch
        # started later, when a ring fills or after an idle return, counts in the requests' time)
        self._start()
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def finish(q, done_t):
            r, outs, started = outstanding.pop(q)
            V, it, cv, sv = outs
            if keep_results:  # out of the launch's result memory, which later jobs reuse
                V, sv = np.array(V), (None if sv is None else np.array(sv, dtype=bool))
            else:
                V = sv = None
            responses[r.rid] = Response(r.rid, V, np.array(it), np.array(cv, dtype=bool), r.arrival, started,
                                        done_t, self.launches - 1, sv)
            self.backend.release(q)

        def drain():
            # every job the launch started has its results when stop returns; after an idle
            # return (1), jobs published once its CTAs had left were never started: they go
            # back to the front of the queue, for the next launch
            idle = self.backend.stop() == 1
            t = now()
            flags = self.backend.flags()
            redo = []
            for q in sorted(outstanding):
                if flags[q] and self.backend.done(q):
                    finish(q, t)
                elif idle:
                    redo.append(outstanding.pop(q)[0])
                else:
                    raise RuntimeError(f"stream launch stopped with job {q} unfinished")
            pending.extendleft(reversed(redo))

        try:
            i = 0
            while i < len(reqs) or pending or outstanding:
                t = now()
                while i < len(reqs) and (not realtime or reqs[i].arrival <= t):
                    pending.append(reqs[i])
                    i += 1
                busy = False
                if pending and not self.backend.alive():  # the launch reached its idle limit
                    drain()
                    self._start()
                while pending:
                    r = pending[0]
                    sub = self._submit(r)
                    if sub is None:
                        if outstanding and not self.backend.full():
                            break  # staging / result memory held by running jobs: retry as they finish
                        drain()  # the launch's ring is full: finish it and start the next
                        self._start()
                        sub = self._submit(r)
                        if sub is None:
                            raise RuntimeError(f"request {r.rid} does not fit an empty launch (raise its limits)")
                    pending.popleft()
                    outstanding[sub[0]] = (r, sub[1], now())
                    busy = True
                if outstanding:
                    flags = self.backend.flags()
                    ready = [q for q in outstanding if flags[q]]
                    if ready:
                        t = now()
                        for q in ready:
                            if self.backend.done(q):  # (an acquire fence before the results are read)
                                finish(q, t)
                        busy = True
                    elif not self.backend.alive():  # ended at its idle limit before these jobs started
                        drain()
                        self._start()
                        busy = True
                if not busy:
                    wait = 2e-5
                    if realtime and i < len(reqs) and not outstanding:
                        wait = max(wait, min(reqs[i].arrival - now(), 0.002))
                    time.sleep(wait)
        finally:
            if outstanding:
                drain()
            else:
                self.backend.stop()
        return [responses[r.rid] for r in requests]
