"""Seeded synthetic workloads of the traversal benchmark.

The reference publishes no benchmark scenes, so the traversal workload is a
procedural triangle soup and two ray families:

* ``triangle_soup(n, seed)`` — n equilateral triangles, centroids uniform in
  the unit cube, edge length U(0.001, 0.01), orientation a uniform random
  rotation (normalised Gaussian quaternion).  Vertices are not shared.
* ``primary_rays(w, h)`` — pinhole rays of a thin-lens camera with lens
  radius 0 at (0.5, -1, 0.5) looking along +y, 45 degree field of view, one ray
  through each pixel centre (the camera formula of
  src/shader/camera.glsl:62-77 with u.xy = 0.5).
* ``incoherent_rays(...)`` — secondary rays from the closest-hit points of the
  primary set, cosine-distributed about the geometric normal on the side the
  primary ray came from, origin offset 1e-4 along the new direction; primary
  misses are replaced by a uniform origin in the cube with a uniform direction.
* ``shadow_tmax(n, seed)`` — any-hit distances U(0, 1).
"""
from __future__ import annotations

import numpy as np

TRAVERSAL_SEEDS = {1 << 20: 101, 1 << 22: 104, 1 << 24: 116}


def _rng(seed: int) -> np.random.Generator:
    return np.random.default_rng(seed)


def triangle_soup(n: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """(vertices float32 (3n, 3), indices uint32 (3n,))."""
    rng = _rng(seed)
    centroid = rng.random((n, 3))
    edge = rng.uniform(0.001, 0.01, n)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    rot = np.empty((n, 3, 3))
    rot[:, 0, 0] = 1 - 2 * (y * y + z * z)
    rot[:, 0, 1] = 2 * (x * y - z * w)
    rot[:, 0, 2] = 2 * (x * z + y * w)
    rot[:, 1, 0] = 2 * (x * y + z * w)
    rot[:, 1, 1] = 1 - 2 * (x * x + z * z)
    rot[:, 1, 2] = 2 * (y * z - x * w)
    rot[:, 2, 0] = 2 * (x * z - y * w)
    rot[:, 2, 1] = 2 * (y * z + x * w)
    rot[:, 2, 2] = 1 - 2 * (x * x + y * y)
    ang = np.array([0.0, 2 * np.pi / 3, 4 * np.pi / 3])
    local = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)], axis=1)  # unit circumradius
    radius = edge / np.sqrt(3.0)
    verts = centroid[:, None, :] + radius[:, None, None] * np.einsum("nij,kj->nki", rot, local)
    vertices = verts.reshape(-1, 3).astype(np.float32)
    indices = np.arange(3 * n, dtype=np.uint32)
    return vertices, indices


def primary_rays(width: int, height: int, pos=(0.5, -1.0, 0.5), fov_deg: float = 45.0):
    """(origins, dirs) float32 (w*h, 3), row-major over pixels (y, x)."""
    pos = np.asarray(pos, np.float32)
    front = np.array([0.0, 1.0, 0.0], np.float32)
    right = np.array([1.0, 0.0, 0.0], np.float32)
    up = np.array([0.0, 0.0, 1.0], np.float32)
    tan_fov = np.float32(np.tan(np.radians(fov_deg * 0.5)))
    asp = np.float32(width / height)
    ys, xs = np.meshgrid(np.arange(height, dtype=np.float32), np.arange(width, dtype=np.float32), indexing="ij")
    u = (xs / np.float32(width) + np.float32(0.5) / np.float32(width)) * 2 - 1
    v = (ys / np.float32(height) + np.float32(0.5) / np.float32(height)) * 2 - 1
    px = (u * asp * tan_fov).reshape(-1)
    py = (v * tan_fov).reshape(-1)
    d = right[None] * px[:, None] + up[None] * py[:, None] + front[None] * np.float32(1.0)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(pos, d.shape).copy()
    return o.astype(np.float32), d.astype(np.float32)


def _triangle_normals(vertices: np.ndarray, indices: np.ndarray, prim: np.ndarray) -> np.ndarray:
    tri = indices.reshape(-1, 3)[prim]
    a, b, c = vertices[tri[:, 0]], vertices[tri[:, 1]], vertices[tri[:, 2]]
    n = np.cross(b.astype(np.float64) - a, c.astype(np.float64) - a)
    return n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)


def incoherent_rays(vertices, indices, origins, dirs, hit_id, hit_t, seed: int):
    """Secondary rays from the primary hits (see the module docstring)."""
    rng = _rng(seed)
    n = origins.shape[0]
    hit_id = np.asarray(hit_id)
    hit_t = np.asarray(hit_t, np.float64)
    hit = hit_id >= 0
    out_o = np.empty((n, 3), np.float64)
    out_d = np.empty((n, 3), np.float64)
    # cosine-distributed direction about the normal facing the incoming side
    k = int(hit.sum())
    if k:
        ng = _triangle_normals(vertices, indices, hit_id[hit])
        d_in = dirs[hit].astype(np.float64)
        flip = np.sum(ng * d_in, axis=1) > 0
        ng[flip] = -ng[flip]
        u1, u2 = rng.random(k), rng.random(k)
        r = np.sqrt(u1)
        phi = 2 * np.pi * u2
        local = np.stack([r * np.cos(phi), r * np.sin(phi), np.sqrt(np.maximum(0.0, 1 - u1))], axis=1)
        t = np.where(np.abs(ng[:, 2:3]) > 0.999, np.array([[0.0, 1.0, 0.0]]), np.array([[0.0, 0.0, 1.0]]))
        bvec = np.cross(ng, t)
        bvec /= np.linalg.norm(bvec, axis=1, keepdims=True)
        tvec = np.cross(bvec, ng)
        wd = tvec * local[:, 0:1] + bvec * local[:, 1:2] + ng * local[:, 2:3]
        wd /= np.linalg.norm(wd, axis=1, keepdims=True)
        p = origins[hit].astype(np.float64) + d_in * hit_t[hit][:, None]
        out_o[hit] = p + wd * 1e-4
        out_d[hit] = wd
    m = n - k
    if m:
        out_o[~hit] = rng.random((m, 3))
        g = rng.standard_normal((m, 3))
        out_d[~hit] = g / np.linalg.norm(g, axis=1, keepdims=True)
    return out_o.astype(np.float32), out_d.astype(np.float32)


def shadow_tmax(n: int, seed: int) -> np.ndarray:
    return _rng(seed).random(n).astype(np.float32)
