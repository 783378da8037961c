"""Host-side pieces that need no GPU: the synthetic inputs, the planner and the device
schedule (executed serially on the CPU), the C ABI's exported symbols, the multi-rank
case sharding."""

import ctypes as C
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from oracle import cpu
from p3s_gb300 import _lib
from p3s_gb300.synthetic import grid_118, grid_2000, lanes, make_grid, timeseries_injections

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_synthetic_sizes_match_the_configs(grid118, grid2000):
    assert (grid118.n, grid118.n_branch, grid118.nnz, len(grid118.pv), len(grid118.pq)) == (118, 186, 490, 19, 98)
    assert (grid2000.n, grid2000.n_branch, grid2000.nnz, len(grid2000.pv), len(grid2000.pq)) == (
        2000, 3000, 8000, 300, 1699)
    # the branch stamps sum to the Ybus
    Y = np.zeros(grid2000.nnz, dtype=complex)
    np.add.at(Y, grid2000.stamp_pos.ravel(), grid2000.stamp.ravel())
    assert np.abs(Y - grid2000.Yx).max() < 1e-10
    # deterministic
    g2 = grid_118(0)
    assert np.array_equal(g2.Yx, grid118.Yx) and np.array_equal(g2.pv, grid118.pv)


def test_timeseries_and_lanes(grid118):
    S = timeseries_injections(grid118, 48)
    assert S.shape == (118, 48) and S.flags.c_contiguous
    # hourly generation follows the hourly load (balanced dispatch)
    ratio = S[grid118.pv].real.sum(axis=0) / -S[grid118.pq].real.sum(axis=0)
    assert np.allclose(ratio, grid118.p_gen.sum() / grid118.p_load.sum())
    off = lanes(8760, 1216)
    assert off[0] == 0 and off[-1] == 8760 and len(off) == 1217 and set(np.diff(off)) <= {7, 8}


def _selftest(g, workers, seed=1, chain_cap=1.0):
    L = _lib.load()
    rng = np.random.default_rng(seed)
    Vm = np.abs(g.V0) * (1 + 0.02 * rng.standard_normal(g.n))
    Va = np.angle(g.V0) + 0.05 * rng.standard_normal(g.n)
    dx = np.zeros(2 * g.n)
    shape = np.zeros(7, np.int32)
    msg = C.create_string_buffer(256)
    Yx = np.ascontiguousarray(g.Yx)
    S = np.ascontiguousarray(g.Sbus)
    rc = L.gbpf_plan_selftest(g.n, _lib.i32(g.Yp), _lib.i32(g.Yj), _lib.cview(Yx), g.nnz, _lib.i32(g.pv), len(g.pv),
                              _lib.i32(g.pq), len(g.pq), workers, _lib.d(Vm), _lib.d(Va), _lib.cview(S), _lib.d(dx),
                              _lib.i32(shape), msg, 256, float(chain_cap))
    assert rc == 0, msg.value
    d = cpu.Solver(g.Yp, g.Yj, g.Yx, g.pv, g.pq).debug_J_at(g.Sbus, Vm * np.exp(1j * Va))
    J = sp.csc_matrix((d["Jx"], d["Ji"], d["Jp"]), shape=(d["m"], d["m"]))
    x = spl.spsolve(J, -d["F"])
    pvpq = np.r_[g.pv, g.pq]
    ref = np.zeros((g.n, 2))
    ref[pvpq, 0] = x[: len(pvpq)]
    ref[g.pq, 1] = x[len(pvpq):]
    return np.abs(dx.reshape(-1, 2) - ref).max() / max(1.0, np.abs(ref).max()), shape


@pytest.mark.parametrize("workers", [1, 16, 64, 1024])
def test_block_schedule_solves_the_power_flow_jacobian(workers):
    """The device's 2x2-block LU schedule, executed serially with a race check per level,
    solves what scipy solves (the reference's test_plan_solves_power_flow_jacobian)."""
    for g in (grid_118(), grid_2000()):
        err, shape = _selftest(g, workers)
        assert err < 1e-9, err


@pytest.mark.parametrize("cap", [0.0, 0.25, 0.5, 2.0])
def test_block_schedule_with_other_chain_caps(cap):
    """Schedules with the chain segments cut finer, coarser or not at all (the tuner's knob)
    keep every dependency (the per-level race check) and solve the same system."""
    for g in (grid_118(), grid_2000()):
        err, _ = _selftest(g, 64, chain_cap=cap)
        assert err < 1e-9, err


def test_block_schedule_large_and_irregular():
    err, shape = _selftest(make_grid(20000, seed=3), 64)
    assert err < 1e-9
    err, shape = _selftest(make_grid(30, seed=4), 32)
    assert err < 1e-9


def test_library_exports_every_declared_symbol():
    """libgbpf.so loads without a GPU and exports every function include/gbpf.h declares."""
    L = _lib.load()
    hdr = open(os.path.join(ROOT, "include", "gbpf.h")).read()
    names = set(re.findall(r"\b(gbpf_[a-z0-9_]+)\s*\(", hdr))
    names -= {n for n in names if n.endswith("_t")}
    assert len(names) >= 18
    for n in sorted(names):
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, n
    assert L.gbpf_version() >= 100
    assert L.gbpf_device_count() >= 0


def test_case_sharding_covers_every_case_once():
    from bench import shard

    for B, W in ((8760, 1), (8760, 2), (3001, 4), (5, 8)):
        seen = np.concatenate([np.arange(*shard(B, r, W)) for r in range(W)])
        assert np.array_equal(np.sort(seen), np.arange(B))


def _header_structs():
    """Field names of every `typedef struct NAME { ... } NAME;` in include/gbpf.h, in order."""
    hdr = open(os.path.join(ROOT, "include", "gbpf.h")).read()
    hdr = re.sub(r"/\*.*?\*/", " ", hdr, flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (\w+) \{(.*?)\} \1;", hdr, flags=re.S):
        fields = []
        for decl in body.split(";"):
            for piece in decl.split(","):
                ids = re.findall(r"[A-Za-z_]\w*", piece)
                if ids:
                    fields.append(ids[-1])
        out[name] = fields
    return out


@pytest.mark.parametrize("cname, py", [("gbpf_params", "Params"), ("gbpf_info", "Info"), ("gbpf_stats", "Stats"),
                                       ("gbpf_job", "Job")])
def test_ctypes_structs_follow_the_header(cname, py, tmp_path):
    """The ctypes mirrors of the C ABI's structs: same fields in the same order, and the same
    offsets and size as the C compiler lays them out."""
    import shutil
    import subprocess

    fields = _header_structs()[cname]
    S = getattr(_lib, py)
    assert [f for f, _ in S._fields_] == fields
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "gbpf.h"\nint main(void) {\n'
                   + "".join(f'    printf("%zu\\n", offsetof({cname}, {f}));\n' for f in fields)
                   + f'    printf("%zu\\n", sizeof({cname}));\n    return 0;\n}}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == [getattr(S, f).offset for f in fields] + [C.sizeof(S)]


def test_pooled_result_blocks_are_reused_once_dropped(monkeypatch):
    """Page-locked result blocks (faked here by plain host buffers): a dropped array's block
    serves the next request of about its size; views keep it, copies do not; blocks beyond
    the pool's limit are released."""
    from p3s_gb300 import solver

    live, freed = {}, []

    class FakeLib:
        def gbpf_host_alloc(self, nbytes):
            buf = (C.c_char * nbytes)()
            live[C.addressof(buf)] = buf
            return C.addressof(buf)

        def gbpf_host_free(self, ptr):
            freed.append(ptr)

    fake = FakeLib()
    monkeypatch.setattr(_lib, "load", lambda: fake)
    pool = solver._HostPool(keep=40_000)
    monkeypatch.setattr(solver, "_HOST_POOL", pool)
    a = solver.pooled_empty((100, 10), np.complex128)  # 16,000 bytes
    assert type(a) is np.ndarray and a.flags.c_contiguous and len(live) == 1
    a[:] = 1.0
    pa = a.ctypes.data
    del a
    assert pool._held == 16_000
    b = solver.pooled_empty((90, 10), np.complex128)  # fits the dropped block: reused
    assert b.ctypes.data == pa and len(live) == 1 and pool._held == 0
    c = solver.pooled_empty((10, 10), np.complex128)  # far smaller than any free block: a new one
    assert len(live) == 2
    d = b[:, :3].copy()
    v = c[:, 1:]
    del b, c
    assert pool._held == 16_000  # b's block is back; c's is held by its view
    del v
    assert pool._held == 17_600 and d.base is None
    e = solver.pooled_empty((200, 10), np.complex128)  # 32,000 bytes: new
    del e  # 49,600 would exceed the 40,000-byte limit: released
    assert freed == [list(live)[2]] and pool._held == 17_600


def test_outage_lists():
    """Case-group outage lists (ptr, idx) as the outage jobs take them; the full N-1 sweep's
    lists made directly equal the generic ones."""
    from p3s_gb300 import contingency

    ptr, idx = contingency.outage_lists([[], [3], [1, 2], []])
    assert ptr.tolist() == [0, 0, 1, 3, 3] and idx.tolist() == [3, 1, 2]
    assert ptr.dtype == np.int32 and idx.dtype == np.int32
    for m in (0, 1, 7, 3000):
        a = contingency.single_outage_lists(m)
        b = contingency.outage_lists([[]] + [[e] for e in range(m)])
        assert all(np.array_equal(x, y) and x.dtype == y.dtype for x, y in zip(a, b))


def _shaped_grid(kind: str, n: int, all_pv: bool = False):
    """A small grid of a given shape (bus 0 the slack): 'chain' (a deep elimination tree),
    'star' (one hub column as long as the grid), 'mesh' (a square lattice: fill), with series
    impedance 0.01 + 0.1j per line and alternating PV / PQ buses (or PV only)."""
    from types import SimpleNamespace

    from p3s_gb300.synthetic import build_ybus

    if kind == "chain":
        f, t = np.arange(n - 1), np.arange(1, n)
    elif kind == "star":
        f, t = np.zeros(n - 1, int), np.arange(1, n)
    else:
        k = int(round(np.sqrt(n)))
        n = k * k
        idx = np.arange(n).reshape(k, k)
        f = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
        t = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    y = 1.0 / (0.01 + 0.1j)
    stamp = np.tile(np.array([y + 0.01j, -y, -y, y + 0.01j]), (len(f), 1))
    Yp, Yj, Yx, _ = build_ybus(n, f.astype(np.int32), t.astype(np.int32), stamp)
    rest = np.arange(1, n, dtype=np.int32)
    pv = rest if all_pv else np.ascontiguousarray(rest[::2])
    pq = np.zeros(0, np.int32) if all_pv else np.ascontiguousarray(rest[1::2])
    rng = np.random.default_rng(n)
    S = np.zeros(n, complex)
    S[1:] = -0.01 * (1 + rng.random(n - 1)) - 0.005j
    return SimpleNamespace(n=n, Yp=Yp, Yj=Yj, Yx=Yx, nnz=len(Yj), pv=pv, pq=pq, V0=np.ones(n, complex), Sbus=S)


@pytest.mark.parametrize("kind", ["chain", "star", "mesh"])
@pytest.mark.parametrize("workers", [1, 16, 1024])
def test_block_schedule_on_shaped_grids(kind, workers):
    """Deep elimination trees, one long hub column (split into chain segments) and lattice
    fill: the schedule, executed serially with its race check, solves what scipy solves."""
    for n, all_pv in ((2, False), (3, True), (400, False), (400, True)):
        err, shape = _selftest(_shaped_grid(kind, n, all_pv), workers)
        assert err < 1e-9, (kind, n, all_pv, err)


def test_no_cpu_fallback_without_a_device(grid118):
    """Without a visible CUDA device every product entry point raises (no silent CPU path)."""
    if _lib.load().gbpf_device_count() > 0:
        pytest.skip("a CUDA device is visible")
    from p3s_gb300 import nr_klu
    from p3s_gb300.cuda.nr_polar_solver import PolarNewtonSolverCUDA
    from p3s_gb300.group import GpuGroup
    from p3s_gb300.solver import GpuSolver

    g = grid118
    args = (g.Yp, g.Yj, g.Yx, g.pv, g.pq)
    for make in (lambda: GpuSolver(*args), lambda: nr_klu.Solver(*args), lambda: PolarNewtonSolverCUDA(*args),
                 lambda: nr_klu.solve_single(g.Yp, g.Yj, g.Yx, g.Sbus, g.V0, g.pv, g.pq), lambda: GpuGroup()):
        with pytest.raises(RuntimeError):
            make()


def test_autotune_pins_the_fastest_shape_and_chain_cap():
    """The tuner's selection: every (threads, slots, chain cap) candidate timed (best of its
    runs, the first run discarded as the shape's build), the fastest pinned -- the shape for the
    batch's size class, the cap for the solver -- and every timing returned."""
    from p3s_gb300 import autotune

    class FakeSolver:
        def __init__(self):
            self.chain_cap, self.shape, self.stats, self.pinned = 1.0, None, {}, []

        def set_chain_cap(self, cap):
            self.chain_cap = cap

        def set_shape(self, units, nt, g):
            self.shape = (units, nt, g)
            self.pinned.append(self.shape)

    s = FakeSolver()
    cost = {(512, 32, 1.0): 10.0, (512, 32, 0.5): 9.5, (1024, 16, 1.0): 11.0, (1024, 16, 0.5): 12.0}
    runs = []

    def run():
        key = (s.shape[1], s.shape[2], s.chain_cap)
        runs.append(key)
        # the first run of a candidate is slow (it builds the schedule): the tuner must not keep it
        s.stats = {"kernel_ms": cost[key] + (100.0 if runs.count(key) == 1 else 0.0)}

    choice, timings = autotune.tune(s, 8760, run, candidates=((512, 32), (1024, 16)), chain_caps=(1.0, 0.5), reps=2)
    assert choice == (512, 32, 0.5) and timings == cost
    assert s.chain_cap == 0.5 and s.shape == (8760, 512, 32)
    assert len(runs) == 4 * 3
