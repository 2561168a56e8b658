"""Known-answer tests of the oracle traversal (CPU).

Each case follows a branch of src/shader/intersection.glsl: the unscaled
|det| < 1e-6 rejection (:76), the double-sided sign flip (:83-87), the
axis-dominant and near-zero-component branches of boxHit (:236-319), the
`boxDist > dist` prune and the strict `t < dist` closest update (:409-418).
"""
from __future__ import annotations

import numpy as np

import oracle


def _scene(tris):
    v = np.asarray(tris, np.float32).reshape(-1, 3)
    idx = np.arange(v.shape[0], dtype=np.uint32)
    b, h, _ = oracle.bvh_build(v, idx)
    return b, h, v, idx


def _trace(scene, o, d, tmax=None, any_hit=False):
    b, h, v, idx = scene
    o = np.asarray(o, np.float32).reshape(-1, 3)
    d = np.asarray(d, np.float32).reshape(-1, 3)
    return oracle.trace(b, h, v, idx, o, d, tmax=tmax, any_hit=any_hit, nthreads=1)


UNIT = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]


def test_axis_ray_hits_and_distance_is_exact():
    sc = _scene(UNIT)
    hid, t, vis, tst = _trace(sc, [0.25, 0.25, 2.0], [0, 0, -1])
    assert hid[0] == 0 and t[0] == np.float32(2.0) and tst[0] == 1


def test_double_sided():
    sc = _scene(UNIT)
    hid, t, _, _ = _trace(sc, [0.25, 0.25, -3.0], [0, 0, 1])
    assert hid[0] == 0 and t[0] == np.float32(3.0)


def test_miss_returns_minus_one_and_1e8():
    sc = _scene(UNIT)
    hid, t, _, _ = _trace(sc, [2.0, 2.0, 1.0], [0, 0, -1])
    assert hid[0] == -1 and t[0] == np.float32(1e8)


def test_small_triangle_rejected_by_unscaled_det_epsilon():
    # |det| = |ab . (d x ac)| = 1e-3 * 1e-3 for a right triangle of legs 1e-3
    # facing the ray: 1e-6 is not < 1e-6 ... legs 9e-4 give 8.1e-7 < 1e-6.
    small = (np.asarray(UNIT, np.float64) * 9e-4).tolist()
    sc = _scene(small)
    hid, _, _, tst = _trace(sc, [2e-4, 2e-4, 1.0], [0, 0, -1])
    assert tst[0] == 1 and hid[0] == -1
    big = (np.asarray(UNIT, np.float64) * 2e-3).tolist()
    hid, _, _, _ = _trace(_scene(big), [2e-4, 2e-4, 1.0], [0, 0, -1])
    assert hid[0] == 0


def test_closest_of_stacked_triangles_and_tie_goes_to_first_in_order():
    stack = [[[0, 0, z], [1, 0, z], [0, 1, z]] for z in (0.0, 0.5, 0.25)]
    sc = _scene([p for tri in stack for p in tri])
    hid, t, _, _ = _trace(sc, [0.2, 0.2, 1.0], [0, 0, -1])
    assert hid[0] == 1 and t[0] == np.float32(0.5)
    # two identical triangles: the strict '<' keeps the first one in table order
    sc = _scene(UNIT + UNIT)
    b, h, v, idx = sc
    hid, _, _, _ = _trace(sc, [0.2, 0.2, 1.0], [0, 0, -1])
    face = 4  # cubemapFace(-dir) for dir = (0, 0, -1): -dir.z > 0 -> face 4
    order = [p for p in h[face, :, 1] if p >= 0]
    assert hid[0] == order[0]


def test_any_hit_respects_tmax_strictly():
    sc = _scene(UNIT)
    o, d = [0.25, 0.25, 2.0], [0, 0, -1]
    occ, _, _, _ = _trace(sc, o, d, tmax=np.array([2.0], np.float32), any_hit=True)
    assert occ[0] == 0  # t == tmax is not < tmax
    occ, _, _, _ = _trace(sc, o, d, tmax=np.array([2.0001], np.float32), any_hit=True)
    assert occ[0] == 1


def test_general_branch_with_zero_direction_component():
    # direction in the y-z plane: |d.x| < 1e-6 takes the near-zero branch
    tris = [[-1, 0.5, 0.5], [1, 0.5, 0.5], [0, 0.5, 1.5]]  # in the plane y = 0.5
    sc = _scene(tris)
    d = np.array([0.0, 1.0, 1.0], np.float32)
    d /= np.linalg.norm(d)
    hid, t, _, _ = _trace(sc, [0.0, 0.0, 0.25], d)
    assert hid[0] == 0
    assert abs(float(t[0]) - 0.5 * np.sqrt(2)) < 1e-6


def test_empty_scene_misses():
    v = np.zeros((0, 3), np.float32)
    idx = np.zeros(0, np.uint32)
    hid, t, vis, tst = oracle.trace(np.zeros((0, 6), np.float32), np.zeros((6, 0, 3), np.int32), v, idx,
                                    np.zeros((2, 3), np.float32), np.ones((2, 3), np.float32))
    assert np.all(hid == -1) and np.all(t == np.float32(1e8)) and np.all(vis == 0)
