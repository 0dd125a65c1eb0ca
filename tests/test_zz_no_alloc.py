"""The allocation-free RayQueue sort (wf_ray_schedule_static).

It exists for callers that may not allocate device memory while they run:
code inside a framework that owns the device heap, loops under a
no-allocation rule, work prepared during stream capture.  They pass their own
device buffers; the sort's scratch is a fixed device array inside the library.

This file is collected last, so a failure here comes after every other test.
It must pass alone in a fresh process and after the other tests: the array
keeps the previous call's contents, and the entry point must not depend on
them.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rays(rng, n):
    o = rng.uniform(-12, 12, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[: n // 100, 1] = 0.0
    o[n // 2: n // 2 + n // 50] = o[n // 2]  # runs of equal keys: the order must stay stable
    return o, d


def test_static_schedule_matches_allocating_entry_point(wf):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    lib = wf.load_library()
    ctx = wf.Context(0)
    bmin = np.array([-10, -10, -10], np.float32)
    bmax = np.array([10, 10, 10], np.float32)
    rng = np.random.default_rng(4242)
    # two calls in a row, different sizes: the second must not see the first's data
    for n in (300_000, 123_457):
        o, d = _rays(rng, n)
        want_perm, want_keys = ctx.ray_schedule(o, d, bmin, bmax)
        cols = [torch.from_numpy(np.ascontiguousarray(a[:, k])).cuda() for a in (o, d) for k in range(3)]
        perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        keys = torch.zeros((n,), dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        rc = lib.wf_ray_schedule_static(None, n, *[c.data_ptr() for c in cols], wf.ptr(bmin), wf.ptr(bmax),
                                        perm.data_ptr(), keys.data_ptr())
        assert rc == wf.WF_OK
        torch.cuda.synchronize()
        assert np.array_equal(perm.cpu().numpy(), want_perm)
        assert np.array_equal(keys.cpu().numpy().view(np.uint64), want_keys)
    # Its defining property: once the library's module is loaded (the calls
    # above), a call takes no device memory, so the device's free memory is
    # the same before and after it.
    free_before = torch.cuda.mem_get_info()[0]
    rc = lib.wf_ray_schedule_static(None, n, *[c.data_ptr() for c in cols], wf.ptr(bmin), wf.ptr(bmax),
                                    perm.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == wf.WF_OK
    assert torch.cuda.mem_get_info()[0] == free_before
    assert np.array_equal(perm.cpu().numpy(), want_perm)
    ctx.close()


def test_static_schedule_matches_the_reference_golden_permutation(wf):
    """RayQueue::schedule's permutation and keys as the reference's own code
    computed them (tests/golden/ray_schedule.npz, include/scheduling/
    RayQueue.h:135-179), through the allocation-free entry point."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    from conftest import GOLDEN

    g = np.load(GOLDEN / "ray_schedule.npz")
    lib = wf.load_library()
    n = len(g["perm"])
    cols = [torch.from_numpy(np.ascontiguousarray(g[a][:, k])).cuda() for a in ("o", "d") for k in range(3)]
    perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    keys = torch.zeros((n,), dtype=torch.int64, device="cuda")
    bmin = np.ascontiguousarray(g["bmin"], np.float32)
    bmax = np.ascontiguousarray(g["bmax"], np.float32)
    torch.cuda.synchronize()
    rc = lib.wf_ray_schedule_static(None, n, *[c.data_ptr() for c in cols], wf.ptr(bmin), wf.ptr(bmax),
                                    perm.data_ptr(), keys.data_ptr())
    torch.cuda.synchronize()
    assert rc == wf.WF_OK
    assert np.array_equal(perm.cpu().numpy(), g["perm"])
    assert np.array_equal(keys.cpu().numpy().view(np.uint64), g["keys"])


def test_static_schedule_rejects_sizes_beyond_its_scratch(wf):
    lib = wf.load_library()
    bmin = np.zeros(3, np.float32)
    bmax = np.ones(3, np.float32)
    n = wf.STATIC_SCHEDULE_MAX_RAYS + 1
    rc = lib.wf_ray_schedule_static(None, n, *([1] * 6), wf.ptr(bmin), wf.ptr(bmax), 1, None)
    assert wf.ERRORS[rc] == "WF_ERR_CAPACITY"
