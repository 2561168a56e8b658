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


# ---------------------------------------------------------------------------
# Cornell-style path-tracing scene
# ---------------------------------------------------------------------------
def _quad(p0, p1, p2, p3, n):
    v = np.array([p0, p1, p2, p3], np.float64)
    nn = np.tile(np.asarray(n, np.float64), (4, 1))
    return v, nn, np.array([0, 1, 2, 0, 2, 3], np.int64)


def _box(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    faces = [
        ((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1), (0, -1, 0)),
        ((x1, y1, z0), (x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (0, 1, 0)),
        ((x0, y1, z0), (x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (-1, 0, 0)),
        ((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1), (1, 0, 0)),
        ((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1), (0, 0, 1)),
        ((x0, y1, z0), (x1, y1, z0), (x1, y0, z0), (x0, y0, z0), (0, 0, -1)),
    ]
    return [_quad(*f) for f in faces]


def _uv_sphere(center, radius, segments=32, rings=16):
    c = np.asarray(center, np.float64)
    verts, idx = [], []
    for i in range(rings + 1):
        th = np.pi * i / rings
        for j in range(segments + 1):
            ph = 2 * np.pi * j / segments
            verts.append((np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)))
    verts = np.array(verts)
    row = segments + 1
    for i in range(rings):
        for j in range(segments):
            a, b, cc, d = i * row + j, (i + 1) * row + j, (i + 1) * row + j + 1, i * row + j + 1
            if i != 0:
                idx += [a, b, d]
            if i != rings - 1:
                idx += [b, cc, d]
    return c + radius * verts, verts.copy(), np.array(idx, np.int64)


def cornell_scene(seed: int = 1, width: int = 256, height: int = 256, sampler: int = 1):
    """Seeded Cornell-style box: 5 Lambertian walls with albedo U(0.2, 0.8)^3,
    one area-light quad of power 15 under the ceiling, two axis-aligned boxes
    and two 32x16 UV spheres (about 2k triangles); one sphere carries the only
    principled material (roughness U(0.1, 0.9), metallic in {0, 1}).  Z is up,
    the camera looks along +y into the open side of the box."""
    from .scene import LAMBERTIAN, PRINCIPLED, SceneData, mat_tex, material

    rng = np.random.default_rng(seed)
    mats, parts = [], []  # parts: (verts, normals, idx, material index)

    def add(mesh_list, mat_rec):
        mats.append(mat_rec)
        m = len(mats) - 1
        for v, n, i in mesh_list:
            parts.append((v, n, i, m))

    walls = [
        ((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0), (0, 0, 1)),      # floor
        ((-1, 1, 2), (1, 1, 2), (1, -1, 2), (-1, -1, 2), (0, 0, -1)),     # ceiling
        ((-1, 1, 0), (1, 1, 0), (1, 1, 2), (-1, 1, 2), (0, -1, 0)),       # back
        ((-1, -1, 0), (-1, 1, 0), (-1, 1, 2), (-1, -1, 2), (1, 0, 0)),    # left
        ((1, 1, 0), (1, -1, 0), (1, -1, 2), (1, 1, 2), (-1, 0, 0)),       # right
    ]
    for w in walls:
        add([_quad(*w)], material(LAMBERTIAN, base_color=rng.uniform(0.2, 0.8, 3)))
    add(_box((-0.65, 0.15, 0.0), (-0.15, 0.65, 1.2)), material(LAMBERTIAN, base_color=rng.uniform(0.2, 0.8, 3)))
    add(_box((0.125, -0.575, 0.0), (0.575, -0.125, 0.45)), material(LAMBERTIAN, base_color=rng.uniform(0.2, 0.8, 3)))
    add([_uv_sphere((-0.45, -0.45, 0.3), 0.3)],
        material(PRINCIPLED, base_color=rng.uniform(0.2, 0.8, 3), roughness=rng.uniform(0.1, 0.9),
                 metallic=float(rng.integers(0, 2))))
    add([_uv_sphere((0.5, 0.5, 0.25), 0.25)], material(LAMBERTIAN, base_color=rng.uniform(0.2, 0.8, 3)))

    ov, on, oi, om = [], [], [], []
    base = 0
    for v, n, i, m in parts:
        ov.append(v)
        on.append(n)
        oi.append(i + base)
        om += [mat_tex(m)] * (i.size // 3)
        base += v.shape[0]
    lv, ln, li = _quad((-0.3, -0.3, 1.98), (0.3, -0.3, 1.98), (0.3, 0.3, 1.98), (-0.3, 0.3, 1.98), (0, 0, -1))
    return SceneData(
        obj_vertices=np.concatenate(ov), obj_normals=np.concatenate(on), obj_indices=np.concatenate(oi),
        obj_mat_tex=np.array(om, np.int32), materials=np.stack(mats),
        light_vertices=lv, light_normals=ln, light_indices=li, light_first=np.array([0, 2], np.uint32),
        light_power=np.array([[15.0, 15.0, 15.0]]), film=(width, height), cam_pos=(0.0, -3.4, 1.0),
        cam_angle=(0.0, 0.0, 0.0), cam_fov=40.0, cam_lens_radius=0.0, cam_focal_dist=1.0, sampler=sampler,
    ).normalized()


def sky_environment(width: int, height: int, seed: int = 2, sun_dir=(0.4, -0.3, 0.866), peak_over_mean=1e3):
    """Procedural equirectangular environment (rows = polar angle from +z):
    a sky gradient plus a Gaussian sun lobe scaled so that peak/mean is about
    `peak_over_mean`.  Returns float32 (height, width, 3)."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    phi = np.pi * v[:, None]
    theta = 2 * np.pi * u[None, :]
    d = np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi) * np.ones_like(theta)], -1)
    up = np.clip(d[..., 2], -1, 1)
    sky = np.stack([0.3 + 0.2 * up, 0.45 + 0.25 * up, 0.7 + 0.3 * up], -1)
    sky = np.clip(sky, 0.02, None) * (1.0 + 0.02 * rng.standard_normal(sky.shape[:2]))[..., None]
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    lobe = np.exp((d @ s - 1.0) / 0.0004)
    sky_mean = sky.mean()
    img = sky + lobe[..., None] * np.array([1.0, 0.95, 0.85])
    peak = img.max()
    scale = (peak_over_mean * img.mean() - sky_mean) if peak > 0 else 0.0
    img = sky + lobe[..., None] * np.array([1.0, 0.95, 0.85]) * max(scale, 1.0)
    return np.clip(img, 0.0, None).astype(np.float32)


def _sphere_batch(centers, radii, segments, rings):
    """Vertices/normals/indices of many UV spheres at once."""
    unit_v, unit_n, unit_i = _uv_sphere((0.0, 0.0, 0.0), 1.0, segments, rings)
    k = centers.shape[0]
    nv = unit_v.shape[0]
    verts = centers[:, None, :] + radii[:, None, None] * unit_v[None]
    norms = np.broadcast_to(unit_n[None], (k, nv, 3))
    idx = unit_i[None, :] + (np.arange(k) * nv)[:, None]
    return verts.reshape(-1, 3), norms.reshape(-1, 3), idx.reshape(-1)


def city_scene(seed: int = 2, width: int = 1920, height: int = 1080, grid: int = 64, n_spheres: int = 2000,
               sphere_segments: int = 64, sphere_rings: int = 16, env_size=(2048, 1024), n_lights: int = 8):
    """Seeded procedural city: a grid x grid block of boxes with heights
    lognormal(0, 0.5) on a ground plane, n_spheres UV spheres (64x16 by
    default, about 4M triangles in total) scattered above it, 16 principled
    materials with every parameter uniform in its range, a sky-gradient plus
    sun environment (peak/mean about 1e3) and n_lights small emissive quads
    (the light and triple integrators sample light triangles)."""
    from .scene import PRINCIPLED, SceneData, mat_tex, material

    rng = np.random.default_rng(seed)
    mats = [material(PRINCIPLED, base_color=rng.uniform(0, 1, 3), roughness=rng.uniform(),
                     subsurface=rng.uniform(), metallic=rng.uniform(), specular=rng.uniform(),
                     specular_tint=rng.uniform(), sheen=rng.uniform(), sheen_tint=rng.uniform(),
                     clearcoat=rng.uniform(), clearcoat_gloss=rng.uniform()) for _ in range(16)]
    vs, ns, ids, mt = [], [], [], []
    base = 0

    def add(v, n, i, m):
        nonlocal base
        vs.append(np.asarray(v, np.float64))
        ns.append(np.asarray(n, np.float64))
        ids.append(np.asarray(i, np.int64) + base)
        mt.append(np.full(len(i) // 3, mat_tex(m), np.int32))
        base += len(v)

    # ground
    g = float(grid)
    v, n, i = _quad((0, 0, 0), (g, 0, 0), (g, g, 0), (0, g, 0), (0, 0, 1))
    add(v, n, i, int(rng.integers(16)))
    # buildings: one box per cell, 12 triangles each
    heights = rng.lognormal(0.0, 0.5, (grid, grid))
    foot = rng.uniform(0.55, 0.85, (grid, grid))
    bm = rng.integers(0, 16, (grid, grid))
    for gx in range(grid):
        for gy in range(grid):
            h, f = heights[gx, gy], foot[gx, gy]
            cx, cy = gx + 0.5, gy + 0.5
            bv, bn, bi = [], [], []
            off = 0
            for qv, qn, qi in _box((cx - f / 2, cy - f / 2, 0.0), (cx + f / 2, cy + f / 2, h)):
                bv.append(qv)
                bn.append(qn)
                bi.append(qi + off)
                off += 4
            add(np.concatenate(bv), np.concatenate(bn), np.concatenate(bi), int(bm[gx, gy]))
    # spheres, grouped by material
    centers = np.stack([rng.uniform(0, g, n_spheres), rng.uniform(0, g, n_spheres),
                        rng.uniform(2.0, 6.0, n_spheres)], 1)
    radii = rng.uniform(0.1, 0.45, n_spheres)
    sm = rng.integers(0, 16, n_spheres)
    for m in range(16):
        sel = sm == m
        if sel.any():
            v, n, i = _sphere_batch(centers[sel], radii[sel], sphere_segments, sphere_rings)
            add(v, n, i, m)
    # emissive quads facing down, above the city
    lv, ln, li, lf, lp = [], [], [], [0], []
    for k in range(n_lights):
        x, y = rng.uniform(4, g - 4, 2)
        z = 8.0
        s = 0.5
        qv, qn, qi = _quad((x - s, y - s, z), (x + s, y - s, z), (x + s, y + s, z), (x - s, y + s, z), (0, 0, -1))
        li.append(qi + 4 * k)
        lv.append(qv)
        ln.append(qn)
        lf.append(lf[-1] + 2)
        lp.append([2.0e4, 1.8e4, 1.5e4])
    return SceneData(
        obj_vertices=np.concatenate(vs), obj_normals=np.concatenate(ns), obj_indices=np.concatenate(ids),
        obj_mat_tex=np.concatenate(mt), materials=np.stack(mats),
        light_vertices=np.concatenate(lv), light_normals=np.concatenate(ln), light_indices=np.concatenate(li),
        light_first=np.array(lf, np.uint32), light_power=np.array(lp), film=(width, height),
        cam_pos=(-6.0, -6.0, 14.0), cam_angle=(45.0, -28.0, 0.0), cam_fov=50.0, sampler=1,
        env_rgb=sky_environment(env_size[0], env_size[1], seed=seed + 1), env_rotation=0.0,
    ).normalized()


def sphere_box_scene(seed: int, n_tris: int, width: int, height: int, sampler: int = 1):
    """Cornell box plus enough 32x16 UV spheres (960 triangles each) scattered
    inside it to reach about `n_tris` triangles, materials drawn per sphere
    (Lambertian or principled)."""
    from .scene import LAMBERTIAN, PRINCIPLED, mat_tex, material

    d = cornell_scene(seed=seed, width=width, height=height, sampler=sampler)
    rng = np.random.default_rng(seed + 1000)
    k = max(0, (n_tris - d.obj_indices.size // 3) // 960)
    if k == 0:
        return d
    centers = np.stack([rng.uniform(-0.9, 0.9, k), rng.uniform(-0.9, 0.9, k), rng.uniform(0.1, 1.9, k)], 1)
    radii = rng.uniform(0.02, 0.12, k)
    mats = list(d.materials)
    v, n, i = _sphere_batch(centers, radii, 32, 16)
    base = d.obj_vertices.shape[0]
    per = i.size // 3 // k
    sphere_mat = []
    for j in range(k):
        if rng.uniform() < 0.5:
            mats.append(material(LAMBERTIAN, base_color=rng.uniform(0.2, 0.8, 3)))
        else:
            mats.append(material(PRINCIPLED, base_color=rng.uniform(0.2, 0.8, 3), roughness=rng.uniform(0.1, 0.9),
                                 metallic=float(rng.integers(0, 2))))
        sphere_mat += [mat_tex(len(mats) - 1)] * per
    d.obj_vertices = np.concatenate([d.obj_vertices, v.astype(np.float32)])
    d.obj_normals = np.concatenate([d.obj_normals, n.astype(np.float32)])
    d.obj_indices = np.concatenate([d.obj_indices, (i + base).astype(np.uint32)])
    d.obj_mat_tex = np.concatenate([d.obj_mat_tex, np.array(sphere_mat, np.int32)])
    d.materials = np.stack(mats)
    return d.normalized()


def material_zoo_scene(seed: int = 41, width: int = 64, height: int = 64, sampler: int = 1):
    """The Cornell-style box of :func:`cornell_scene` with every material type:
    Lambertian walls, a metal-workflow tall box (metallic 0.7, roughness 0.4),
    a thin-dielectric short box (ior 1.5), a smooth glass sphere (roughness
    0, ior 1.5) and a rough dielectric sphere (roughness 0.35, ior 1.33)."""
    from .scene import DIELECTRIC, METAL_WORKFLOW, THIN_DIELECTRIC, material

    d = cornell_scene(seed=seed, width=width, height=height, sampler=sampler)
    mats = np.array(d.materials, np.float32, copy=True)
    # cornell_scene material order: 5 walls, tall box, short box, principled sphere, sphere
    mats[5] = material(METAL_WORKFLOW, base_color=(0.9, 0.7, 0.4), roughness=0.4, metallic=0.7)
    mats[6] = material(THIN_DIELECTRIC, base_color=(0.95, 0.95, 0.9), ior=1.5)
    mats[7] = material(DIELECTRIC, base_color=(1.0, 1.0, 1.0), roughness=0.0, ior=1.5)
    mats[8] = material(DIELECTRIC, base_color=(0.9, 1.0, 0.95), roughness=0.35, ior=1.33)
    d.materials = mats
    return d.normalized()


def texture_images(seed: int = 51):
    """Three seeded 8-bit sRGB RGB images of different sizes (a 40x24
    two-colour checkerboard, a 17x31 noise image and a 64x64 gradient with a
    grid), top row first."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:24, 0:40]
    c0, c1 = rng.integers(0, 256, 3), rng.integers(0, 256, 3)
    checker = np.where(((x // 5 + y // 4) % 2)[..., None] == 0, c0, c1).astype(np.uint8)
    noise = rng.integers(0, 256, (17, 31, 3)).astype(np.uint8)
    y, x = np.mgrid[0:64, 0:64]
    grad = np.stack([x * 4, y * 4, 255 - (x + y) * 2], -1)
    grad[(x % 16 == 0) | (y % 16 == 0)] = 255
    return [checker, noise, np.clip(grad, 0, 255).astype(np.uint8)]


def textured_scene(seed: int = 51, width: int = 64, height: int = 64, sampler: int = 1, base: str = "cornell"):
    """A scene with albedo textures: ``base`` is the Cornell-style box
    ("cornell"), the material zoo ("zoo") or the 8-material box of
    :func:`diff_scene` ("diff").  The floor, back and left walls, the tall box
    and the principled sphere are textured (three images of different sizes),
    the other objects keep their material colour.  Texcoords are linear in
    the position and span about [-1.5, 2.5], so they wrap and go negative."""
    from .scene import mat_tex

    make = {"cornell": cornell_scene, "zoo": material_zoo_scene, "diff": diff_scene}[base]
    d = make(seed=seed, width=width, height=height, sampler=sampler)
    if base == "diff":  # diff_scene shares one material between the boxes: map through the object order
        d0 = cornell_scene(seed=seed, width=width, height=height, sampler=sampler)
        objects = d0.obj_mat_tex & 0xFFFF
    else:
        objects = d.obj_mat_tex & 0xFFFF
    rng = np.random.default_rng(seed + 7)
    a, b = rng.uniform(-1.0, 1.0, 3), rng.uniform(-1.0, 1.0, 3)
    p = d.obj_vertices.astype(np.float64)
    d.obj_texcoords = np.stack([p @ a + 0.5, p @ b - 0.25], 1).astype(np.float32)
    # cornell_scene material order: floor, ceiling, back, left, right, tall box, short box, sphere, sphere
    tex_of_object = {0: 0, 2: 1, 3: 2, 5: 1, 7: 2}
    mats = d.obj_mat_tex & 0xFFFF
    d.obj_mat_tex = np.array([mat_tex(int(m), tex_of_object.get(int(o), -1)) for m, o in zip(mats, objects)],
                             np.int32)
    d.textures = texture_images(seed)
    return d.normalized()


def diff_scene(seed: int = 11, width: int = 512, height: int = 512, sampler: int = 1):
    """The Cornell-style box of :func:`cornell_scene` with 8 principled
    materials (5 walls, the two boxes sharing one, the two spheres), each with
    baseColor U(0.2, 0.8)^3, roughness U(0.1, 0.9), metallic U(0, 1),
    specular U(0, 1): 8 * 6 material parameters plus the light's power rgb."""
    from .scene import PRINCIPLED, material, mat_tex

    d = cornell_scene(seed=seed, width=width, height=height, sampler=sampler)
    rng = np.random.default_rng(seed + 1000)
    mats = [material(PRINCIPLED, base_color=rng.uniform(0.2, 0.8, 3), roughness=rng.uniform(0.1, 0.9),
                     metallic=rng.uniform(0.0, 1.0), specular=rng.uniform(0.0, 1.0)) for _ in range(8)]
    # cornell_scene material order: 5 walls, box, box, principled sphere, sphere
    remap = np.array([0, 1, 2, 3, 4, 5, 5, 6, 7], np.int32)
    old = d.obj_mat_tex & 0xFFFF
    d.obj_mat_tex = np.array([mat_tex(int(m)) for m in remap[old]], np.int32)
    d.materials = np.stack(mats)
    return d.normalized()


def perturbed_params(p0: np.ndarray, n_materials: int, seed: int = 12, scale: float = 0.3) -> np.ndarray:
    """Initial guess for inverse rendering: every material parameter moved by
    U(-scale, scale) and clamped to [0.02, 1]; light power unchanged."""
    rng = np.random.default_rng(seed)
    p = np.array(p0, np.float32, copy=True)
    k = 6 * n_materials
    p[:k] = np.clip(p[:k] + rng.uniform(-scale, scale, k).astype(np.float32), 0.02, 1.0)
    return p


def batch_requests(seed: int = 3, n: int = 64):
    """Seeded request list of the batched-serving workload: n scenes with
    log-uniform triangle counts in [1k, 500k], log-uniform square films in
    [128, 1024], spp uniform in {4..64} and depth uniform in {4..8}.
    Returns [(SceneData, spp, params)]."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n):
        tris = int(np.exp(rng.uniform(np.log(1e3), np.log(5e5))))
        side = int(np.exp(rng.uniform(np.log(128), np.log(1024))))
        spp = int(rng.integers(4, 65))
        depth = int(rng.integers(4, 9))
        out.append((sphere_box_scene(seed * 1000 + r, tris, side, side), spp, dict(max_depth=depth)))
    return out
