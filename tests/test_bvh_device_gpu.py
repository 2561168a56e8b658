"""MTBVH built by the CUDA kernels (zgl_accel_build_device) against the
oracle's quickBuild + buildHitTable restatement (src/accelerator/BVH.cpp:
217-345): bounds (every bit, including the sign of zero bounds) and the six
threaded tables are identical, whatever the subtree threshold that splits the
work between the level kernels and the per-warp subtree kernel."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.test_bvh_host import _cases
from zillumgl_gb300 import BVH, ZglError
from zillumgl_gb300.synthetic import incoherent_rays, primary_rays, triangle_soup

pytestmark = pytest.mark.gpu

# 8: nearly every inner node goes through the level kernels; 64: both paths;
# 0: the default threshold (512), small meshes are one warp subtree
THRESHOLDS = (8, 64, 0)


def _export(acc):
    p = acc.export()
    acc.close()
    return p


def _all_cases():
    # the host builder's 300k signed-zero soup stays a host case (the device
    # builder has its own signed-zero grid, 100k and 1M soups)
    yield from (c for c in _cases() if c[0] != "soup_300k_zeros")
    v = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (700, 1))
    yield "identical_2100", v, np.arange(v.shape[0], dtype=np.uint32)
    yield ("soup_100k", *triangle_soup(100_000, 13))


@pytest.mark.parametrize("small", THRESHOLDS)
@pytest.mark.parametrize("name,v,idx", list(_all_cases()), ids=lambda x: x if isinstance(x, str) else "")
def test_device_build_matches_oracle_bitwise(zgl_lib, cuda, name, v, idx, small):
    ob, oh, _ = oracle.bvh_build(v, idx)
    p = _export(BVH(v, idx).build_device(small_threshold=small))
    assert p.bounds.shape == ob.shape
    assert np.array_equal(p.bounds.view(np.uint32), ob.view(np.uint32)), name
    assert np.array_equal(p.hitTable, oh), name


def test_large_mesh_matches_host_builder(zgl_lib, cuda):
    v, idx = triangle_soup(1 << 20, 101)
    host = BVH(v, idx).build_host()
    for small in (0, 256):
        p = _export(BVH(v, idx).build_device(small_threshold=small))
        assert np.array_equal(p.bounds.view(np.uint32), host.bounds.view(np.uint32))
        assert np.array_equal(p.hitTable, host.hitTable)


def test_device_and_pinned_inputs(zgl_lib, cuda):
    import torch

    v, idx = triangle_soup(30_000, 14)
    ref = _export(BVH(v, idx).build())
    tv = torch.from_numpy(v).to(cuda)
    ti = torch.from_numpy(idx.view(np.int32)).to(cuda)
    p = _export(BVH(tv, ti).build_device())
    assert np.array_equal(p.bounds.view(np.uint32), ref.bounds.view(np.uint32))
    assert np.array_equal(p.hitTable, ref.hitTable)
    pv = torch.from_numpy(v).pin_memory()
    pi = torch.from_numpy(idx.view(np.int32)).pin_memory()
    bvh = BVH(v, idx)
    bvh._vertices, bvh._indices = pv.numpy(), pi.numpy().view(np.uint32)
    p = _export(bvh.build_device(small_threshold=64))
    assert np.array_equal(p.bounds.view(np.uint32), ref.bounds.view(np.uint32))
    assert np.array_equal(p.hitTable, ref.hitTable)


def test_traversal_on_device_built_tree(zgl_lib, cuda):
    """Node records and triangle records of the device build give the oracle's
    hits bit for bit (closest and any-hit, coherent and incoherent rays)."""
    import torch

    v, idx = triangle_soup(200_000, 15)
    acc = BVH(v, idx).build_device()
    p = acc.export()
    o, d = primary_rays(96, 96)
    ph, pt, _, _ = oracle.trace(p.bounds, p.hitTable, v, idx, o, d)
    oi, di = incoherent_rays(v, idx, o, d, ph, pt, seed=5)
    for oo, dd in ((o, d), (oi, di)):
        to, td = torch.from_numpy(oo).to(cuda), torch.from_numpy(dd).to(cuda)
        hid, ht = acc.trace_closest(to, td)
        tmax = torch.full((oo.shape[0],), 0.3, device=cuda)
        occ = acc.trace_any(to, td, tmax)
        torch.cuda.synchronize()
        ohid, oht, _, _ = oracle.trace(p.bounds, p.hitTable, v, idx, oo, dd)
        oocc, _, _, _ = oracle.trace(p.bounds, p.hitTable, v, idx, oo, dd, tmax=np.full(oo.shape[0], 0.3,
                                                                                       np.float32), any_hit=True)
        assert np.array_equal(hid.cpu().numpy(), ohid)
        assert np.array_equal(ht.cpu().numpy().view(np.uint32), oht.view(np.uint32))
        assert np.array_equal(occ.cpu().numpy(), oocc)
    acc.close()


def test_empty_and_invalid_meshes(zgl_lib, cuda):
    acc = BVH(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32)).build_device()
    p = _export(acc)
    assert p.bounds.shape == (0, 6)
    v = np.zeros((3, 3), np.float32)
    with pytest.raises(ZglError) as e:
        BVH(v, np.array([0, 1, 7], np.uint32)).build_device()
    assert "out of range" in str(e.value)
    for x in (np.nan, np.inf, 3e8):
        bad = v.copy()
        bad[1, 2] = x
        with pytest.raises(ZglError):
            BVH(bad, np.array([0, 1, 2], np.uint32)).build_device()
    with pytest.raises(ZglError):
        BVH(v, np.array([0, 1, 2], np.uint32)).build_device(small_threshold=5000)
    # the context is still usable after the rejected builds
    p = _export(BVH(*triangle_soup(50, 1)).build_device())
    assert p.bounds.shape == (99, 6)
