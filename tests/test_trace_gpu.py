"""GPU traversal parity: closest-hit ids and distances, any-hit flags and the
per-ray work counters of the CUDA kernels are bit-identical to the oracle
(src/shader/intersection.glsl:367-427 restated on the CPU)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import BVH
from zillumgl_gb300.synthetic import incoherent_rays, primary_rays, shadow_tmax, triangle_soup

pytestmark = pytest.mark.gpu


def _rays_mixed(rng, n):
    """Random rays including axis-aligned and zero-component directions."""
    o = rng.random((n, 3)).astype(np.float32) * 1.2 - 0.1
    d = rng.standard_normal((n, 3))
    k = n // 8
    d[:k] = 0
    d[np.arange(k), rng.integers(0, 3, k)] = rng.choice([-1.0, 1.0], k)      # exact axis rays
    d[k:2 * k, rng.integers(0, 3)] = 0.0                                       # one zero component
    d[2 * k:3 * k] = np.array([1e-7, 1.0, 0.0]) * rng.choice([-1, 1], (k, 3))  # near-axis (> 1 - 1e-6)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def _check_closest(acc, packed, v, idx, o, d, cuda):
    import torch

    to = torch.from_numpy(o).to(cuda)
    td = torch.from_numpy(d).to(cuda)
    hid, ht = acc.trace_closest(to, td)
    torch.cuda.synchronize()
    ohid, oht, ovis, otst = oracle.trace(packed.bounds, packed.hitTable, v, idx, o, d)
    g_id, g_t = hid.cpu().numpy(), ht.cpu().numpy()
    bad = np.nonzero(g_id != ohid)[0]
    assert bad.size == 0, f"{bad.size} hit ids differ, first ray {bad[:5]}"
    assert np.array_equal(g_t.view(np.uint32), oht.view(np.uint32)), "hit distances differ"
    vis, tst = acc.trace_count(to, td)
    assert np.array_equal(vis.cpu().numpy(), ovis) and np.array_equal(tst.cpu().numpy(), otst)
    return g_id, g_t


@pytest.fixture(scope="module")
def soup(zgl_lib, cuda):
    v, idx = triangle_soup(60000, 5)
    acc = BVH(v, idx).build()
    packed = acc.export()
    ob, oh, _ = oracle.bvh_build(v, idx)
    assert np.array_equal(packed.bounds.view(np.uint32), ob.view(np.uint32))
    assert np.array_equal(packed.hitTable, oh)
    yield acc, packed, v, idx
    acc.close()


@pytest.mark.parametrize("schedule", ["auto", "thread_per_ray", "persistent", "prefetch"])
def test_primary_and_incoherent_closest_bit_exact(soup, cuda, schedule):
    acc, packed, v, idx = soup
    acc.set_trace_schedule(schedule)
    try:
        o, d = primary_rays(96, 96)
        hid, ht = _check_closest(acc, packed, v, idx, o, d, cuda)
        assert (hid >= 0).mean() > 0.2
        o2, d2 = incoherent_rays(v, idx, o, d, hid, ht, seed=9)
        _check_closest(acc, packed, v, idx, o2, d2, cuda)
    finally:
        acc.set_trace_schedule("auto")


@pytest.mark.parametrize("schedule", ["auto", "thread_per_ray", "persistent", "prefetch"])
def test_mixed_rays_closest_bit_exact(soup, cuda, schedule):
    acc, packed, v, idx = soup
    acc.set_trace_schedule(schedule)
    try:
        o, d = _rays_mixed(np.random.default_rng(3), 20000)
        _check_closest(acc, packed, v, idx, o, d, cuda)
    finally:
        acc.set_trace_schedule("auto")


@pytest.mark.parametrize("schedule", ["auto", "thread_per_ray", "persistent", "prefetch"])
def test_any_hit_bit_exact(soup, cuda, schedule):
    import torch

    acc, packed, v, idx = soup
    o, d = _rays_mixed(np.random.default_rng(4), 20000)
    tmax = shadow_tmax(o.shape[0], 5)
    acc.set_trace_schedule(schedule)
    try:
        occ = acc.trace_any(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda),
                            torch.from_numpy(tmax).to(cuda)).cpu().numpy()
    finally:
        acc.set_trace_schedule("auto")
    oocc, _, ovis, otst = oracle.trace(packed.bounds, packed.hitTable, v, idx, o, d, tmax=tmax, any_hit=True)
    assert np.array_equal(occ.astype(np.int32), oocc)
    vis, tst = acc.trace_count(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda),
                               torch.from_numpy(tmax).to(cuda), any_hit=True)
    assert np.array_equal(vis.cpu().numpy(), ovis) and np.array_equal(tst.cpu().numpy(), otst)


def _long_rays(rng, n):
    """Rays with one direction component below 1e-6 (boxHit's near-zero
    branch: every box whose slab holds the origin on that axis is entered),
    interleaved with ordinary random rays so that warps mix long and short
    rays."""
    o = rng.random((n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3))
    axis = rng.integers(0, 3, n)
    d[np.arange(n), axis] = rng.choice([-1.0, 1.0], n) * rng.uniform(1e-8, 9e-7, n)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    o2, d2 = _rays_mixed(rng, n)
    oo = np.empty((2 * n, 3), np.float32)
    dd = np.empty((2 * n, 3), np.float32)
    oo[0::2], dd[0::2] = o, d
    oo[1::2], dd[1::2] = o2, d2
    return oo, dd


@pytest.mark.parametrize("schedule", ["auto", "prefetch"])
@pytest.mark.parametrize("n", [4001, 20000])
def test_long_rays_finished_by_the_warp_bit_exact(soup, cuda, schedule, n):
    """Rays that outrun the 256-entry lane budget are finished by their
    warps 32 entries at a time: ids, distances and any-hit flags equal the
    oracle's, with long and short rays in one warp and a partial last warp."""
    import torch

    acc, packed, v, idx = soup
    o, d = _long_rays(np.random.default_rng(41), n // 2)
    o, d = o[:n], d[:n]
    tmax = shadow_tmax(o.shape[0], 42) * 2.0
    vis, _ = acc.trace_count(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda))
    assert int((vis.cpu().numpy() > 256).sum()) >= 10, "too few rays past the lane budget"
    acc.set_trace_schedule(schedule)
    try:
        _check_closest(acc, packed, v, idx, o, d, cuda)
        occ = acc.trace_any(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda),
                            torch.from_numpy(tmax).to(cuda)).cpu().numpy()
    finally:
        acc.set_trace_schedule("auto")
    oocc, _, _, _ = oracle.trace(packed.bounds, packed.hitTable, v, idx, o, d, tmax=tmax, any_hit=True)
    assert np.array_equal(occ.astype(np.int32), oocc)


def test_host_arrays_match_device_arrays(soup, cuda):
    import torch

    acc, packed, v, idx = soup
    o, d = _rays_mixed(np.random.default_rng(6), 5000)
    hid_h, ht_h = acc.trace_closest(o, d)  # numpy: staged through the library
    hid_d, ht_d = acc.trace_closest(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda))
    assert np.array_equal(hid_h, hid_d.cpu().numpy())
    assert np.array_equal(ht_h.view(np.uint32), ht_d.cpu().numpy().view(np.uint32))
    tmax = shadow_tmax(o.shape[0], 1)
    occ_h = acc.trace_any(o, d, tmax)
    occ_d = acc.trace_any(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda),
                          torch.from_numpy(tmax).to(cuda))
    assert np.array_equal(occ_h, occ_d.cpu().numpy())


def test_empty_and_single_triangle_accelerators(zgl_lib, cuda):
    o, d = _rays_mixed(np.random.default_rng(8), 1000)
    empty = BVH(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32)).build()
    hid, ht = empty.trace_closest(o, d)
    assert np.all(hid == -1) and np.all(ht == np.float32(1e8))
    assert not empty.trace_any(o, d, np.ones(1000, np.float32)).any()
    empty.close()
    v = np.array([[0, 0, 0.5], [1, 0, 0.5], [0, 1, 0.5]], np.float32)
    one = BVH(v, np.arange(3, dtype=np.uint32)).build()
    p = one.export()
    hid, ht = one.trace_closest(o, d)
    ohid, oht, _, _ = oracle.trace(p.bounds, p.hitTable, v, np.arange(3, dtype=np.uint32), o, d)
    assert np.array_equal(hid, ohid) and np.array_equal(ht.view(np.uint32), oht.view(np.uint32))
    one.close()


def test_zero_rays_is_a_no_op(soup):
    acc = soup[0]
    hid, ht = acc.trace_closest(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    assert hid.size == 0 and ht.size == 0


def test_full_scale_scene_sampled_rays(zgl_lib, cuda):
    """1M-triangle traversal scene: a sample of its 4096^2 primary rays and of
    the incoherent set, bit-exact against the oracle on the same full tree."""
    import torch

    v, idx = triangle_soup(1 << 20, 101)
    acc = BVH(v, idx).build()
    p = acc.export()
    o, d = primary_rays(4096, 4096)
    rng = np.random.default_rng(0)
    sel = rng.choice(o.shape[0], 8192, replace=False)
    hid, ht = _check_closest(acc, p, v, idx, o[sel], d[sel], cuda)
    o2, d2 = incoherent_rays(v, idx, o[sel], d[sel], hid, ht, seed=1)
    _check_closest(acc, p, v, idx, o2, d2, cuda)
    tmax = shadow_tmax(o2.shape[0], 2)
    occ = acc.trace_any(torch.from_numpy(o2).to(cuda), torch.from_numpy(d2).to(cuda),
                        torch.from_numpy(tmax).to(cuda)).cpu().numpy()
    oocc, _, _, _ = oracle.trace(p.bounds, p.hitTable, v, idx, o2, d2, tmax=tmax, any_hit=True)
    assert np.array_equal(occ.astype(np.int32), oocc)
    acc.close()


def test_host_arrays_equal_device_arrays(soup, cuda):
    """Pinned host arrays are read and written in place by the kernels,
    pageable ones are staged; results equal the device-array call bit for
    bit either way."""
    import torch

    acc, packed, v, idx = soup
    rng = np.random.default_rng(17)
    n = (1 << 21) + 12345
    o, d = _rays_mixed(rng, n)
    tm = rng.random(n).astype(np.float32)
    to, td, tt = (torch.from_numpy(x).to(cuda) for x in (o, d, tm))
    ref_id, ref_t = acc.trace_closest(to, td)
    ref_occ = acc.trace_any(to, td, tt)
    torch.cuda.synchronize()
    ref_id, ref_t, ref_occ = ref_id.cpu().numpy(), ref_t.cpu().numpy(), ref_occ.cpu().numpy()
    for pinned in (False, True):
        ho, hd, ht_ = (torch.from_numpy(x) for x in (o, d, tm))
        hid = torch.empty(n, dtype=torch.int32)
        hdist = torch.empty(n, dtype=torch.float32)
        hocc = torch.empty(n, dtype=torch.uint8)
        if pinned:
            ho, hd, ht_, hid, hdist, hocc = (x.pin_memory() for x in (ho, hd, ht_, hid, hdist, hocc))
        acc.trace_closest(ho, hd, hid, hdist)
        acc.trace_any(ho, hd, ht_, hocc)
        assert np.array_equal(hid.numpy(), ref_id)
        assert np.array_equal(hdist.numpy().view(np.uint32), ref_t.view(np.uint32))
        assert np.array_equal(hocc.numpy(), ref_occ)
