"""A persistent launch of the Newton kernel that takes jobs while it runs (include/gbpf.h,
``gbpf_stream_*``): requests are admitted as CTAs free up, not as whole launches finish.

``GpuStream`` wraps one stream launch: ``start`` launches the kernel for a set of resident
topologies; ``submit`` stages one job (a topology's cases, in the launch's precision or its
own) and appends it to the launch's ring; the kernel writes the job's results straight into
page-locked host arrays and sets the job's flag (``flags`` is a numpy view of the flags);
``stop`` ends the launch once every job it started is done and returns 0, or 1 if its CTAs had
left at their idle limit (no job published for ``idle_seconds``) -- a job whose flag is still
0 then was never started and goes to the next launch. A launch takes at most ``capacity``
jobs (``full``: stop, start again); its staging arena, page-locked input staging and result
memory are reused as jobs complete (``release`` hands a job's memory back once its results
have been read), and ``submit`` returns None while they are held by unfinished jobs.
No reference counterpart: the reference has no serving loop.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .solver import GpuSolver, c128


class _Slab:
    """Page-locked host memory for job results, used as a circular buffer: a job takes one
    block, and blocks are given back in job order once their job's results are consumed."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes) & ~255
        self.ptr = _lib.load().gbpf_host_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError(_lib.last_error())
        self.buf = (C.c_char * self.nbytes).from_address(self.ptr)
        self.reset()

    def reset(self):
        self.head = self.tail = 0
        self.wrapped = False
        self.live = {}      # job -> (begin, end)
        self.order = []     # jobs in allocation order
        self.released = set()

    def take(self, q: int, parts):
        """Views for the (shape, dtype) parts of job q, or None when the slab has no room now."""
        sizes = [(int(np.prod(sh)) * np.dtype(dt).itemsize + 255) & ~255 for sh, dt in parts]
        need = sum(sizes)
        if need > self.nbytes:
            raise ValueError(f"a job's results ({need} bytes) exceed the result memory ({self.nbytes} bytes)")
        if not self.order:
            self.head = self.tail = 0
            self.wrapped = False
        prev = (self.head, self.wrapped)
        at = None
        if not self.wrapped:
            if self.nbytes - self.head >= need:
                at = self.head
            elif self.tail > need:
                at, self.wrapped = 0, True
        elif self.tail - self.head > need:
            at = self.head
        if at is None:
            self.wrapped = prev[1]
            return None
        self._last = (q, prev)
        self.head = at + need
        self.live[q] = (at, at + need)
        self.order.append(q)
        views, off = [], at
        for (sh, dt), nb in zip(parts, sizes):
            cnt = int(np.prod(sh)) * np.dtype(dt).itemsize
            views.append(np.frombuffer(self.buf, dtype=np.uint8, count=cnt, offset=off).view(dt).reshape(sh))
            off += nb
        return views

    def undo(self, q: int):
        """Give back the block just taken for job q (the job was not submitted after all)."""
        last_q, (head, wrapped) = self._last
        assert last_q == q and self.order and self.order[-1] == q
        self.order.pop()
        self.live.pop(q)
        self.head, self.wrapped = head, wrapped

    def release(self, q: int):
        """Job q's results are consumed; blocks go back in job order."""
        self.released.add(q)
        while self.order and self.order[0] in self.released:
            j = self.order.pop(0)
            self.released.discard(j)
            beg, end = self.live.pop(j)
            if self.wrapped and beg < self.tail:
                self.wrapped = False
            self.tail = end

    def __del__(self):
        try:
            _lib.load().gbpf_host_free(self.ptr)
        except Exception:
            pass


class GpuStream:
    def __init__(self, capacity: int = 8192, arena_bytes: int = 8 << 30, result_bytes: int = 4 << 30, ctas: int = 0,
                 slot_budget: int = 8192, input_bytes: int = 0, threads: int = 1024):
        L = _lib.require_device()
        h = L.gbpf_stream_create(int(capacity), int(arena_bytes), int(threads), int(ctas), int(slot_budget))
        if not h:
            raise RuntimeError(_lib.last_error())
        self._h = h
        self.capacity = int(capacity)
        self._slab = _Slab(result_bytes)
        # page-locked staging of the inputs, so that their copies to the device do not wait
        self._in = _Slab(input_bytes or max(256 << 20, result_bytes // 2))
        self._keep = []
        self._flags = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().gbpf_stream_destroy(h)
            except Exception:
                pass
            self._h = None

    def start(self, solvers: list[GpuSolver], params: _lib.Params, idle_seconds: float = 10.0):
        arr = (C.c_void_p * len(solvers))(*[s._h for s in solvers])
        _lib.check(_lib.load().gbpf_stream_start(self._h, len(solvers), arr, C.byref(params), float(idle_seconds)),
                   "stream_start")
        self._slab.reset()
        self._in.reset()
        self._keep = []
        self.submitted = 0
        ptr = _lib.load().gbpf_stream_flags(self._h)
        self._flags = np.ctypeslib.as_array(ptr, shape=(self.capacity,))

    def submit(self, solver: GpuSolver, S, V0, outages=None, reslack: bool = True, precision: str | None = None):
        """Stage one job: S (n,) or (n, T), V0 (n,); outages = (ptr (T+1,), idx) for N-1 cases;
        precision: None (the launch's), "double" or "mixed" (a launch started mixed).
        Returns (index, (V, iterations, converged, served)) -- arrays in page-locked memory that
        the kernel fills -- or None when this launch can take no more."""
        prec = {None: 0, "double": 1, "mixed": 2}[precision]
        n = solver.n
        S = c128(S)
        V0 = c128(V0).ravel()
        if outages is not None:
            optr = np.ascontiguousarray(outages[0], dtype=np.int32)
            oidx = np.ascontiguousarray(outages[1], dtype=np.int32)
            T = len(optr) - 1
        else:
            T = S.shape[1] if S.ndim == 2 else 1
        if S.shape not in ((n, T), (n,)) or V0.shape != (n,):
            raise ValueError("stream job: S must be (n_bus, T) or (n_bus,) and V0 (n_bus,)")
        if self.submitted >= self.capacity:
            return None
        parts = [((n, T), np.complex128), ((T,), np.int32), ((T,), np.uint8)]
        if outages is not None:
            parts.append(((n, T), np.uint8))
        outs = self._slab.take(self.submitted, parts)
        if outs is None:
            return None
        # every input in page-locked memory (a pageable copy would wait for the running launch)
        in_parts = [(S.shape, np.complex128), (V0.shape, np.complex128)]
        if outages is not None:
            in_parts += [(optr.shape, np.int32), ((max(len(oidx), 1),), np.int32)]
        ins = self._in.take(self.submitted, in_parts)
        if ins is None:
            self._slab.undo(self.submitted)
            return None
        ins[0][...] = S
        ins[1][...] = V0
        S, V0 = ins[0], ins[1]
        if outages is not None:
            ins[2][...] = optr
            ins[3][:len(oidx)] = oidx
            optr, oidx = ins[2], ins[3]
        if outages is None:
            outs.append(None)
        J = _lib.Job()
        J.solver = solver._h
        J.n_cases = T
        J.S = S.ctypes.data
        J.s_per_col = int(S.ndim == 2)
        J.V0 = V0.ctypes.data
        J.v0_per_col = 0
        J.V, J.iterations, J.converged = outs[0].ctypes.data, outs[1].ctypes.data, outs[2].ctypes.data
        J.precision = prec
        keep = [S, V0]
        if outages is not None:
            J.out_ptr, J.out_idx, J.reslack = optr.ctypes.data, oidx.ctypes.data, int(bool(reslack))
            J.served = outs[3].ctypes.data
            keep += [optr, oidx]
        q = _lib.load().gbpf_stream_submit(self._h, C.byref(J))
        if q < 0:  # the job was not taken: its blocks are given back
            self._slab.undo(self.submitted)
            self._in.undo(self.submitted)
            if q == -2:
                return None
            _lib.check(-1, "stream_submit")
        assert q == self.submitted
        self.submitted += 1
        self._keep.append(keep)
        return q, tuple(outs)

    def full(self) -> bool:
        """No further job fits this launch's ring (stop and start again)."""
        return self.submitted >= self.capacity

    def release(self, q: int):
        """Job q is done and its results have been read: its staging and result memory may be
        reused."""
        self._slab.release(q)
        self._in.release(q)

    def flags(self) -> np.ndarray:
        return self._flags

    def done(self, q: int) -> bool:
        return _lib.load().gbpf_stream_done(self._h, int(q)) == 1

    def alive(self) -> bool:
        rc = _lib.load().gbpf_stream_alive(self._h)
        _lib.check(0 if rc >= 0 else -1, "stream_alive")
        return rc == 1

    def stop(self) -> int:
        """Wait for every submitted job; 0, or 1 if the launch had reached its idle limit."""
        rc = _lib.load().gbpf_stream_stop(self._h)
        if rc < 0:
            raise RuntimeError(_lib.last_error())
        self._keep = []
        return rc
