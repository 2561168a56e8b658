"""Allocation-free closest-hit entry point (zgl_trace_closest_noalloc).

Callers with a fixed device-memory budget, or whose own pool allocator owns
the device, cannot let the library call cudaMalloc.  The entry point keeps its
scratch in a static device array; this test calls it through the C ABI and
checks that two calls in a row give exactly the hit ids and distances of
zgl_trace_closest and of the oracle (the same bit-exact tolerance as the other
traversal tests) under every trace schedule, for device arrays and for host
arrays, that repeated calls leave the device's free memory unchanged, and that
oversized batches are rejected.  It runs last (file name) and works alone in a
fresh process too.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import BVH
from zillumgl_gb300._lib import ZGL_OK
from zillumgl_gb300.synthetic import incoherent_rays, primary_rays, triangle_soup

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 18


@pytest.mark.parametrize("schedule", ["auto", "thread_per_ray", "persistent", "prefetch"])
def test_noalloc_matches_trace_closest_on_two_calls(zgl_lib, cuda, schedule):
    import torch

    v, idx = triangle_soup(40000, 33)
    acc = BVH(v, idx).build()
    p = acc.export()
    acc.set_trace_schedule(schedule)
    stream = torch.cuda.current_stream().cuda_stream
    o1, d1 = primary_rays(128, 96)
    h1, t1 = acc.trace_closest(o1, d1)
    o2, d2 = incoherent_rays(v, idx, o1, d1, h1, t1, seed=5)
    for o, d in ((o1, d1), (o2, d2)):  # two calls in a row, different rays
        n = o.shape[0]
        to, td = torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda)
        ref_id, ref_t = acc.trace_closest(to, td)
        out_id = torch.full((n,), -7, dtype=torch.int32, device=cuda)
        out_t = torch.full((n,), -7.0, dtype=torch.float32, device=cuda)
        st = zgl_lib.zgl_trace_closest_noalloc(acc.handle, to.data_ptr(), td.data_ptr(), n, out_id.data_ptr(),
                                               out_t.data_ptr(), stream)
        assert st == ZGL_OK, zgl_lib.zgl_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out_id, ref_id)
        assert torch.equal(out_t.view(torch.int32), ref_t.view(torch.int32))
        orc_id, orc_t, _, _ = oracle.trace(p.bounds, p.hitTable, v, idx, o, d)
        assert np.array_equal(out_id.cpu().numpy(), orc_id)
        assert np.array_equal(out_t.cpu().numpy().view(np.uint32), orc_t.view(np.uint32))
    acc.close()


def test_noalloc_calls_leave_free_device_memory_unchanged(zgl_lib, cuda):
    """After a warm-up call (which may reserve the static array), many calls
    with host arrays, which zgl_trace_closest would stage through memory it
    allocates, change the device's free memory by nothing."""
    import torch

    v, idx = triangle_soup(20000, 36)
    acc = BVH(v, idx).build()
    acc.set_trace_schedule("persistent")
    rng = np.random.default_rng(4)
    n = 1 << 17
    o = rng.random((n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    hid = np.zeros(n, np.int32)
    ht = np.zeros(n, np.float32)
    assert zgl_lib.zgl_trace_closest_noalloc(acc.handle, o.ctypes.data, d.ctypes.data, 1, hid.ctypes.data,
                                             ht.ctypes.data, None) == ZGL_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(20):
        st = zgl_lib.zgl_trace_closest_noalloc(acc.handle, o.ctypes.data, d.ctypes.data, n, hid.ctypes.data,
                                               ht.ctypes.data, None)
        assert st == ZGL_OK, zgl_lib.zgl_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    ref_id, _ = acc.trace_closest(o, d)
    assert np.array_equal(hid, ref_id)
    acc.close()


def test_noalloc_host_arrays_two_calls(zgl_lib, cuda):
    v, idx = triangle_soup(20000, 34)
    acc = BVH(v, idx).build()
    rng = np.random.default_rng(3)
    for n in (5000, 3000):  # the second call must not see the first call's staged data
        o = rng.random((n, 3)).astype(np.float32)
        d = rng.standard_normal((n, 3)).astype(np.float32)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        ref_id, ref_t = acc.trace_closest(o, d)
        hid = np.full(n, -7, np.int32)
        ht = np.full(n, -7.0, np.float32)
        st = zgl_lib.zgl_trace_closest_noalloc(acc.handle, o.ctypes.data, d.ctypes.data, n, hid.ctypes.data,
                                               ht.ctypes.data, None)
        assert st == ZGL_OK, zgl_lib.zgl_last_error()
        assert np.array_equal(hid, ref_id)
        assert np.array_equal(ht.view(np.uint32), ref_t.view(np.uint32))
    acc.close()


def test_noalloc_rejects_batches_over_the_limit(zgl_lib, cuda):
    import torch

    v, idx = triangle_soup(1000, 35)
    acc = BVH(v, idx).build()
    n = MAX_RAYS + 1
    o = torch.zeros((n, 3), dtype=torch.float32, device=cuda)
    hid = torch.zeros(n, dtype=torch.int32, device=cuda)
    ht = torch.zeros(n, dtype=torch.float32, device=cuda)
    st = zgl_lib.zgl_trace_closest_noalloc(acc.handle, o.data_ptr(), o.data_ptr(), n, hid.data_ptr(),
                                           ht.data_ptr(), None)
    assert st == 1
    assert b"262144" in zgl_lib.zgl_last_error()
    acc.close()
