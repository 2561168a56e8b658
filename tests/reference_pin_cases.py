"""Cases pinned to the reference's own code (shared by the fixture generator
tests/golden/make_reference_pins.py and the tests that read its output).

* ``FRAME_CASES``: path-tracer frames.  The fixture holds the SHA-256 of the
  frame that the reference's path_integ_naive.glsl, compiled as C++ by
  oracle/glsl_to_cpp.py, renders from the scene's tables; a GPU frame must
  hash to the same value, i.e. equal it bit for bit.
* ``FILM_CASES``: light-tracer and triple-integrator films (small films are
  stored whole; the GPU splats with float atomics, so they are compared
  within 1e-4 per pixel).
* ``SOUPS``: traversal triangle soups whose PackedBVH, as the reference's
  BVH::build() makes it, the fixture records by SHA-256.
* ``TRACE_CASE``: closest-hit and any-hit results of the reference shader's
  bvhHit / bvhTest on a 60k soup with mixed rays.

Every scene is seeded synthetic data made by zillumgl_gb300.synthetic.
"""
from __future__ import annotations

import numpy as np

from zillumgl_gb300 import synthetic as S


def _indep_uniform():
    d = S.cornell_scene(seed=7, width=32, height=16, sampler=0)
    d.env_rgb = S.sky_environment(32, 16, seed=8)
    return d.normalized()


def _env_rr():
    d = S.cornell_scene(seed=14, width=24, height=16)
    d.env_rgb = S.sky_environment(32, 16, seed=3)
    return d.normalized()


def _env_two_lights():
    from tests.test_tables import _multi_light_scene

    return _multi_light_scene(env=True, w=32, h=24)


# name -> (scene factory, integrator params, passes)
FRAME_CASES = {
    "cornell_48x40": (lambda: S.cornell_scene(seed=1, width=48, height=40), dict(max_depth=5), 3),
    "cornell_256_16spp": (lambda: S.cornell_scene(seed=1, width=256, height=256), dict(max_depth=5), 16),
    "rr_reference_schedule": (lambda: S.cornell_scene(seed=6, width=24, height=24),
                              dict(max_depth=6, russian_roulette=1), 2),
    "independent_sampler_uniform_pick": (_indep_uniform, dict(max_depth=4, light_env_uniform_sample=1,
                                                              light_portion=0.3), 2),
    "env_two_lights": (_env_two_lights, dict(max_depth=4), 2),
    "material_zoo": (lambda: S.material_zoo_scene(seed=41, width=48, height=48), dict(max_depth=6), 2),
    "textured_zoo": (lambda: S.textured_scene(seed=57, width=32, height=32, base="zoo"), dict(max_depth=6), 2),
    "diff_scene_64": (lambda: S.diff_scene(seed=11, width=64, height=64), dict(max_depth=6), 4),
    "city_96x54": (lambda: S.city_scene(seed=2, width=96, height=54), dict(max_depth=8, russian_roulette=1), 1),
}

# name -> (kind, scene factory, params, passes, blocks, loops)
FILM_CASES = {
    "light_cornell": ("light", lambda: S.cornell_scene(seed=11, width=40, height=32), dict(max_depth=5), 2, 2, 1),
    "light_zoo_rr": ("light", lambda: S.material_zoo_scene(seed=41, width=32, height=32),
                     dict(max_depth=6, russian_roulette=1), 1, 2, 1),
    "triple_env_rr": ("triple", _env_rr, dict(max_depth=6, russian_roulette=1), 2, 1, 1),
    "triple_cornell_loops": ("triple", lambda: S.cornell_scene(seed=13, width=32, height=24), dict(max_depth=5),
                             2, 1, 2),
}

SOUPS = {"soup_1M": 1 << 20, "soup_4M": 1 << 22, "soup_16M": 1 << 24}

TRACE_CASE = ("soup_60k_mixed", 60000, 5, 20000, 3)  # name, triangles, soup seed, rays, ray seed


def mixed_rays(rng, n):
    """Random rays including exact-axis, one-zero-component and near-axis directions."""
    o = rng.random((n, 3)).astype(np.float32) * 1.2 - 0.1
    d = rng.standard_normal((n, 3))
    k = n // 8
    d[:k] = 0
    d[np.arange(k), rng.integers(0, 3, k)] = rng.choice([-1.0, 1.0], k)
    d[k:2 * k, rng.integers(0, 3)] = 0.0
    d[2 * k:3 * k] = np.array([1e-7, 1.0, 0.0]) * rng.choice([-1, 1], (k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def sha256(*arrays) -> str:
    import hashlib

    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def frame_rgb(frame) -> np.ndarray:
    """(H, W, 3) float32 running sum from an RGBA frame or an RGB film."""
    return np.ascontiguousarray(np.asarray(frame, np.float32)[..., :3])
