"""Host MTBVH build: product builder vs the oracle restatement, bit for bit,
plus the structural invariants of quickBuild/buildHitTable
(src/accelerator/BVH.cpp:217-345)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import BVH
from zillumgl_gb300.synthetic import triangle_soup

LEAF = np.int32(-(2**31))


def _both(v, idx):
    pb = BVH(v, idx).build_host()
    ob, oh, osz = oracle.bvh_build(v, idx)
    return pb, (ob, oh, osz)


def _signed_zero_grid(n=40, seed=3):
    """A height field whose coordinates hold many -0.0 / +0.0 values."""
    rng = np.random.default_rng(seed)
    xs, ys = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n))
    z = np.where(rng.random(xs.shape) < 0.5, 0.0, 0.3 * rng.random(xs.shape))
    v = np.stack([xs.ravel(), ys.ravel(), z.ravel()], 1).astype(np.float32)
    zero = v == 0
    v[zero & (rng.random(v.shape) < 0.5)] = np.float32(-0.0)
    q = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i
            q += [a, a + 1, a + n, a + 1, a + n + 1, a + n]
    return v, np.array(q, np.uint32)


def _cases():
    rng = np.random.default_rng(7)
    yield "soup_2k", *triangle_soup(2000, 11)
    yield "soup_20k", *triangle_soup(20000, 12)
    # shared-vertex grid mesh (indices reuse vertices)
    g = 24
    xs, ys = np.meshgrid(np.linspace(0, 1, g), np.linspace(0, 1, g))
    v = np.stack([xs.ravel(), ys.ravel(), 0.1 * np.sin(6 * xs.ravel())], 1).astype(np.float32)
    q = []
    for j in range(g - 1):
        for i in range(g - 1):
            a = j * g + i
            q += [a, a + 1, a + g, a + 1, a + g + 1, a + g]
    yield "grid", v, np.array(q, np.uint32)
    # degenerate: identical centroids (zero-width extent -> bucket 0 path)
    v = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (9, 1))
    yield "identical", v, np.arange(27, dtype=np.uint32)
    # collinear centroids along one axis with duplicates
    v = rng.random((300, 3)).astype(np.float32)
    v[:, 1:] = 0.5
    yield "collinear", v, rng.integers(0, 300, 3 * 77).astype(np.uint32)
    for n in (1, 2, 3, 4, 5):
        vv, ii = triangle_soup(n, 100 + n)
        yield f"tiny{n}", vv, ii
    # negative zeros and coincident coordinates
    v = np.array([[-0.0, 0, 0], [0.0, 1, 0], [1, -0.0, 0], [0, 0, -0.0], [0, 0, 0.0], [1, 1, 1]], np.float32)
    yield "signed_zero", v, np.array([0, 1, 2, 3, 4, 5, 1, 2, 3, 0, 4, 5], np.uint32)
    yield ("signed_zero_grid", *_signed_zero_grid())
    # large enough for the multi-threaded top nodes (>= 2^18 triangles), with
    # 5% of the coordinates set to -0.0 / +0.0
    v, idx = triangle_soup(300_000, 13)
    z = np.random.default_rng(14).random(v.shape) < 0.05
    v = v.copy()
    v[z] = np.where(np.random.default_rng(15).random(int(z.sum())) < 0.5, np.float32(-0.0), np.float32(0.0))
    yield "soup_300k_zeros", v, idx


@pytest.mark.parametrize("name,v,idx", list(_cases()), ids=lambda x: x if isinstance(x, str) else "")
def test_host_build_matches_oracle_bitwise(zgl_lib, name, v, idx):
    pb, (ob, oh, _) = _both(v, idx)
    assert pb.bounds.shape == ob.shape
    assert np.array_equal(pb.bounds.view(np.uint32), ob.view(np.uint32)), name
    assert np.array_equal(pb.hitTable, oh), name


@pytest.mark.parametrize("name,v,idx", list(_cases()), ids=lambda x: x if isinstance(x, str) else "")
def test_hit_table_invariants(name, v, idx):
    bounds, hit, sizes = oracle.bvh_build(v, idx)
    ntri = idx.size // 3
    M = 2 * ntri - 1
    assert bounds.shape == (M, 6) and hit.shape == (6, M, 3)
    leaves = sizes < 0
    assert leaves.sum() == ntri
    assert sorted((sizes[leaves] ^ LEAF).tolist()) == list(range(ntri))
    for f in range(6):
        nodes, prims, miss = hit[f, :, 0], hit[f, :, 1], hit[f, :, 2]
        assert sorted(nodes.tolist()) == list(range(M))          # every node once
        assert np.all(miss > np.arange(M)) and np.all(miss <= M)  # forward links
        assert (prims >= 0).sum() == ntri
        assert sorted(prims[prims >= 0].tolist()) == list(range(ntri))
        # leaves skip exactly one entry; inner nodes skip their subtree
        assert np.all(miss[prims >= 0] == np.arange(M)[prims >= 0] + 1)
    # every node box encloses its triangle(s)
    tri = v[idx.reshape(-1, 3)]
    lo, hi = tri.min(1), tri.max(1)
    lp = sizes[leaves] ^ LEAF
    assert np.array_equal(bounds[leaves, :3], lo[lp]) and np.array_equal(bounds[leaves, 3:], hi[lp])
    assert np.all(bounds[0, :3] <= lo.min(0)) and np.all(bounds[0, 3:] >= hi.max(0))


def test_empty_mesh(zgl_lib):
    pb = BVH(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32)).build_host()
    assert pb.bounds.shape == (0, 6) and pb.hitTable.shape == (6, 0, 3)


def test_face_order_follows_centroid_comparison():
    # Two triangles separated along x: face 0 (X+) visits the larger-x child first.
    v = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [5, 0, 0], [5.1, 0, 0], [5, 0.1, 0]], np.float32)
    _, hit, _ = oracle.bvh_build(v, np.arange(6, dtype=np.uint32))
    assert hit[0, 1, 1] == 1 and hit[1, 1, 1] == 0


def test_signed_zero_bounds_are_exercised():
    v, idx = _signed_zero_grid()
    ob, _, _ = oracle.bvh_build(v, idx)
    neg = np.signbit(ob) & (ob == 0)
    pos = ~np.signbit(ob) & (ob == 0)
    assert neg.sum() > 10 and pos.sum() > 10
