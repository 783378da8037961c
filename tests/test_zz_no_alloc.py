"""gbpf_islands_device_static: islanding on caller-owned device buffers with static scratch.

Compared bit for bit with gbpf_islands (the allocating host-pointer entry point) on two
calls in a row; the second call runs a smaller grid, so it starts on scratch that still
holds the first call's contents. Collected last so it also runs after every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(grid, groups):
    from p3s_gb300 import contingency

    batch = contingency.build_batch(grid, groups=groups)
    ptr, idx = batch.outages
    is_slack = np.zeros(grid.n, dtype=np.uint8)
    is_slack[np.asarray(grid.ref, dtype=np.int64)] = 1
    prio = np.zeros(grid.n)
    prio[grid.pv] = grid.p_gen[grid.pv]
    return batch, dict(f=np.ascontiguousarray(batch.f, dtype=np.int32), t=np.ascontiguousarray(batch.t, dtype=np.int32),
                       live=np.ascontiguousarray(batch.live, dtype=np.uint8), ptr=ptr, idx=idx, is_slack=is_slack,
                       prio=prio)


def _static_call(n, a, reslack, L, idx=None):
    import torch

    from p3s_gb300 import _lib

    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in a.items()}
    if idx is not None:
        d["idx"] = torch.from_numpy(idx).to(dev)
    if d["idx"].numel() == 0:
        d["idx"] = torch.zeros(1, dtype=torch.int32, device=dev)
    lab = torch.full((n, L), -7, dtype=torch.int32, device=dev)
    sv = torch.full((n, L), 9, dtype=torch.uint8, device=dev)
    rb = torch.full((n, L), -7, dtype=torch.int32, device=dev)
    ni = torch.full((L,), -7, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = _lib.load().gbpf_islands_device_static(
        n, len(a["f"]), d["f"].data_ptr(), d["t"].data_ptr(), d["live"].data_ptr(), L, d["ptr"].data_ptr(),
        d["idx"].data_ptr(), int(a["ptr"][-1]), d["is_slack"].data_ptr(), d["prio"].data_ptr(), int(reslack),
        lab.data_ptr(), sv.data_ptr(), rb.data_ptr(), ni.data_ptr(), stream)
    return rc, (lab.cpu().numpy(), sv.cpu().numpy().astype(bool), rb.cpu().numpy(), ni.cpu().numpy())


def test_static_scratch_islands_match_allocating_entry_two_calls():
    from p3s_gb300 import _lib, contingency
    from p3s_gb300.synthetic import grid_118, grid_2000

    _lib.require_device()
    g2k = grid_2000()
    rng = np.random.default_rng(5)
    # single and double outages of the 2,000-bus grid (islands and re-slacked islands appear)
    groups = [[]] + [[b] for b in range(g2k.n_branch)] + [sorted(rng.choice(g2k.n_branch, 2, replace=False).tolist())
                                                          for _ in range(200)]
    g118 = grid_118()
    runs = [(g2k, groups, True), (g118, None, True)]
    for grid, grp, reslack in runs:
        batch, a = _inputs(grid, grp)
        L = len(batch.groups)
        want = contingency.islands(batch, reslack, a["prio"])
        rc, got = _static_call(grid.n, a, reslack, L)
        assert rc == 0, _lib.last_error()
        for w, x in zip(want, got):
            assert np.array_equal(w, x)
    # reslack off on the same 118-bus cases: unserved islands stay unserved, labels unchanged
    batch, a = _inputs(g118, None)
    want = contingency.islands(batch, False, a["prio"])
    rc, got = _static_call(g118.n, a, False, len(batch.groups))
    assert rc == 0, _lib.last_error()
    for w, x in zip(want, got):
        assert np.array_equal(w, x)


def test_static_scratch_call_allocates_no_device_memory():
    """The property the entry point exists for: with its inputs and outputs already on the
    device, a call leaves the device's free memory where it was (a cudaMalloc of the
    driver's 2 MiB granularity or more would show) and the caching allocator untouched."""
    import torch

    from p3s_gb300 import _lib
    from p3s_gb300.synthetic import grid_2000

    L_ = _lib.require_device()
    g = grid_2000()
    batch, a = _inputs(g, [[]] + [[b] for b in range(400)])
    L = len(batch.groups)
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in a.items()}
    lab = torch.empty((g.n, L), dtype=torch.int32, device=dev)
    sv = torch.empty((g.n, L), dtype=torch.uint8, device=dev)
    rb = torch.empty((g.n, L), dtype=torch.int32, device=dev)
    ni = torch.empty((L,), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def call():
        return L_.gbpf_islands_device_static(
            g.n, len(a["f"]), d["f"].data_ptr(), d["t"].data_ptr(), d["live"].data_ptr(), L, d["ptr"].data_ptr(),
            d["idx"].data_ptr(), int(a["ptr"][-1]), d["is_slack"].data_ptr(), d["prio"].data_ptr(), 1,
            lab.data_ptr(), sv.data_ptr(), rb.data_ptr(), ni.data_ptr(), stream)

    assert call() == 0, _lib.last_error()  # warmed up: scratch address looked up, module loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    reserved0 = torch.cuda.memory_reserved(dev)
    for _ in range(3):
        assert call() == 0, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_reserved(dev) == reserved0


def test_static_scratch_rejects_oversize_and_bad_outages():
    from p3s_gb300 import _lib
    from p3s_gb300.synthetic import grid_118

    L_ = _lib.require_device()
    big = 65537
    rc = L_.gbpf_islands_device_static(big, 0, None, None, None, 1, None, None, 0, None, None, 0, None, None, None,
                                       None, None)
    assert rc != 0 and "exceeds the static scratch maximum of 65536" in _lib.last_error()
    g = grid_118()
    batch, a = _inputs(g, [[0], [1]])
    bad = a["idx"].copy()
    bad[1] = g.n_branch + 3  # an outage index past the branch list: reported, never used
    rc, _ = _static_call(g.n, a, True, 2, idx=bad)
    assert rc != 0 and "outage index out of range" in _lib.last_error()
    # the scratch is usable again after the rejected call
    rc, got = _static_call(g.n, a, True, 2)
    assert rc == 0, _lib.last_error()
