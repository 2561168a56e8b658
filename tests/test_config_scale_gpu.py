"""Parity at the benchmark configurations themselves, not reduced cases.

* Traversal (1M / 4M / 16M triangle soups, seeds 101 / 104 / 116): the
  device-built PackedBVH equals the oracle's quickBuild + buildHitTable bit
  for bit and hashes to the PackedBVH of the reference's own BVH::build()
  (tests/golden/reference_pins.json), and every one of the 2^24 rays of each of the four ray sets the
  benchmark traces (coherent primary and incoherent; closest-hit and any-hit)
  gives the oracle's hit id, distance, occlusion flag and per-ray visit / test
  counters bit for bit (src/shader/intersection.glsl:367-427).
* Cornell box at 256^2, 16 spp, depth 5 (the plain path-tracer
  configuration): every pixel of the 16-sample frame against the oracle,
  within 1e-4 relative and in fact bit for bit; the single-pass and
  multi-pass schedules give the same frame.
* City at 1920x1080 (3.9M triangles, 2048x1024 environment, 16 principled
  materials, depth 8, Russian roulette from depth 3): 4096 sampled pixels of
  two path-tracer passes bit for bit; the light tracer (32 and 203 blocks of
  1536 paths) and the triple integrator (64 blocks) within 1e-4 on a
  480x270 film of the same scene.
* Differentiable configuration (8 principled materials, 512^2, 32 spp,
  depth 6): the forward image of 2048 sampled pixels bit for bit, and the
  51 gradients of a loss on those pixels against the FP64 oracle adjoint.
"""
from __future__ import annotations

import gc
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from tests.reference_pin_cases import sha256
from zillumgl_gb300 import BVH
from zillumgl_gb300.synthetic import (TRAVERSAL_SEEDS, city_scene, cornell_scene, diff_scene, incoherent_rays,
                                      primary_rays, shadow_tmax, triangle_soup)

pytestmark = pytest.mark.gpu

PINS = json.loads((Path(__file__).resolve().parent / "golden" / "reference_pins.json").read_text())
REL_TOL = 1e-4
GRAD_ABS = 2e-3
GRAD_REL = 1e-3


def _same_bits(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def _first_diff(a, b):
    bad = np.nonzero(a != b)[0]
    return f"{bad.size} rays differ, first {bad[:5].tolist()}"


@pytest.mark.parametrize("size", ["1M", "4M", "16M"])
def test_traversal_configuration_all_rays(zgl_lib, cuda, size):
    import torch

    N = {"1M": 1 << 20, "4M": 1 << 22, "16M": 1 << 24}[size]
    seed = TRAVERSAL_SEEDS[N]
    v, idx = triangle_soup(N, seed)
    acc = BVH(v, idx).build_device()
    packed = acc.export()
    ob, oh, _ = oracle.bvh_build(v, idx)
    assert _same_bits(packed.bounds, ob), "device-built bounds differ from the oracle's quickBuild"
    assert np.array_equal(packed.hitTable, oh), "device-built hit tables differ from the oracle's buildHitTable"
    del ob, oh
    assert sha256(packed.bounds, packed.hitTable) == PINS["soups"][f"soup_{size}"]["sha256"], \
        "device-built PackedBVH differs from the reference's BVH::build()"
    n = 4096 * 4096
    o_p, d_p = primary_rays(4096, 4096)
    sets = []
    to, td = torch.from_numpy(o_p).to(cuda), torch.from_numpy(d_p).to(cuda)
    hid, ht = acc.trace_closest(to, td)
    torch.cuda.synchronize()
    g_id, g_t = hid.cpu().numpy(), ht.cpu().numpy()
    r_id, r_t, r_vis, r_tst = oracle.trace(packed.bounds, packed.hitTable, v, idx, o_p, d_p)
    assert np.array_equal(g_id, r_id), f"primary closest: {_first_diff(g_id, r_id)}"
    assert _same_bits(g_t, r_t), "primary closest: hit distances differ"
    sets.append(("primary closest", to, td, None, r_vis, r_tst))
    o_i, d_i = incoherent_rays(v, idx, o_p, d_p, r_id, r_t, seed=seed + 1)
    del hid, ht, g_id, g_t, r_t
    ti, tdi = torch.from_numpy(o_i).to(cuda), torch.from_numpy(d_i).to(cuda)
    hid, ht = acc.trace_closest(ti, tdi)
    torch.cuda.synchronize()
    g_id, g_t = hid.cpu().numpy(), ht.cpu().numpy()
    r_id2, r_t2, r_vis2, r_tst2 = oracle.trace(packed.bounds, packed.hitTable, v, idx, o_i, d_i)
    assert np.array_equal(g_id, r_id2), f"incoherent closest: {_first_diff(g_id, r_id2)}"
    assert _same_bits(g_t, r_t2), "incoherent closest: hit distances differ"
    sets.append(("incoherent closest", ti, tdi, None, r_vis2, r_tst2))
    del hid, ht, g_id, g_t, r_t2
    # any-hit: the camera sits one unit before the cube, so primary shadow distances are 1 + U(0, 1)
    for name, o, d, oh_, dh_, tm in (("primary any", to, td, o_p, d_p, 1.0 + shadow_tmax(n, seed + 2)),
                                     ("incoherent any", ti, tdi, o_i, d_i, shadow_tmax(n, seed + 3))):
        ttm = torch.from_numpy(tm).to(cuda)
        occ = acc.trace_any(o, d, ttm).cpu().numpy()
        r_occ, _, r_v, r_t_ = oracle.trace(packed.bounds, packed.hitTable, v, idx, oh_, dh_, tmax=tm, any_hit=True)
        assert np.array_equal(occ.astype(np.int32), r_occ), f"{name}: {_first_diff(occ.astype(np.int32), r_occ)}"
        sets.append((name, o, d, ttm, r_v, r_t_))
    for name, o, d, ttm, r_v, r_t_ in sets:
        vis, tst = acc.trace_count(o, d, ttm, any_hit=ttm is not None)
        assert np.array_equal(vis.cpu().numpy(), r_v), f"{name}: visit counters differ"
        assert np.array_equal(tst.cpu().numpy(), r_t_), f"{name}: triangle-test counters differ"
    assert (r_id >= 0).mean() > 0.05  # the rays do reach the soup (a sanity check, not a parity one)
    acc.close()
    del sets, to, td, ti, tdi
    gc.collect()
    torch.cuda.empty_cache()


def test_cornell_configuration_full_frame(zgl_lib, cuda):
    from zillumgl_gb300.scene import PathIntegrator, Scene

    data = cornell_scene(seed=1, width=256, height=256)
    params = dict(max_depth=5)
    sc = Scene(data)
    multi = PathIntegrator(sc, **params)
    multi.render_passes(16)
    f_multi, spp = multi.get_frame()
    assert spp == 16
    single = PathIntegrator(sc, **params)
    for _ in range(16):
        single.render_one_pass()
    f_single, _ = single.get_frame()
    assert _same_bits(f_multi, f_single), "multi-pass and single-pass frames differ"
    ref = oracle.OracleScene(data, sc.export("sobol"), params).render_pt(np.arange(256 * 256), 16).reshape(256, 256, 3)
    got = f_multi[..., :3]
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6)
    assert rel.max() <= REL_TOL, f"max rel err {rel.max():.3g}"
    bit_diff = int(np.sum(np.any(got.view(np.uint32) != ref.view(np.uint32), axis=-1)))
    assert bit_diff == 0, f"{bit_diff} pixels differ in some bit (within 1e-4)"
    assert ref.mean() > 0.05
    multi.close()
    single.close()
    sc.close()


CITY_PARAMS = dict(max_depth=8, russian_roulette=1, rr_start_depth=3)


@pytest.fixture(scope="module")
def city_crop(zgl_lib, cuda):
    """The city scene on a 480x270 film (same geometry, materials, environment and lights)."""
    from zillumgl_gb300.scene import Scene

    data = city_scene(seed=2, width=480, height=270)
    sc = Scene(data)
    orc = oracle.OracleScene(data, sc.export("sobol"), CITY_PARAMS)
    yield data, sc, orc
    sc.close()


def test_city_configuration_path_tracer_sampled_pixels(zgl_lib, cuda):
    from zillumgl_gb300.scene import PathIntegrator, Scene

    data = city_scene(seed=2)
    W, H = data.film
    assert (W, H) == (1920, 1080)
    sc = Scene(data)
    integ = PathIntegrator(sc, **CITY_PARAMS)
    integ.render_one_pass()
    integ.render_one_pass()
    frame, spp = integ.get_frame()
    assert spp == 2
    pix = np.sort(np.random.default_rng(2024).choice(W * H, 4096, replace=False)).astype(np.int32)
    ref = oracle.OracleScene(data, sc.export("sobol"), CITY_PARAMS).render_pt(pix, 2)
    got = frame[..., :3].reshape(-1, 3)[pix]
    bad = np.nonzero(np.any(got.view(np.uint32) != ref.view(np.uint32), axis=1))[0]
    assert bad.size == 0, f"{bad.size} of 4096 pixels differ, first pixel {pix[bad[0]]}: {got[bad[0]]} vs {ref[bad[0]]}"
    assert ref.mean() > 0.0
    integ.close()
    sc.close()


def _film_close(got, ref):
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-5)
    worst = np.unravel_index(np.argmax(rel), rel.shape)
    assert rel.max() <= REL_TOL, f"max rel {rel.max():.3g} at {worst}"
    assert ref.sum() > 0


@pytest.mark.parametrize("blocks", [32, 203])
def test_city_light_tracer(city_crop, blocks):
    from zillumgl_gb300.scene import LightIntegrator

    data, sc, orc = city_crop
    params = dict(CITY_PARAMS, blocks_per_pass=blocks)
    integ = LightIntegrator(sc, **params)
    integ.render_one_pass()
    frame, _ = integ.get_frame()
    integ.close()
    _film_close(frame[..., :3], orc.render_lt(1, blocks=blocks))


def test_city_triple_integrator(city_crop):
    from zillumgl_gb300.scene import TripleIntegrator

    data, sc, orc = city_crop
    params = dict(CITY_PARAMS, blocks_per_pass=64)
    integ = TripleIntegrator(sc, **params)
    integ.render_one_pass()
    frame, _ = integ.get_frame()
    integ.close()
    _film_close(frame[..., :3], orc.render_triple(1, blocks=64))


def test_diff_configuration_sampled_pixels(zgl_lib, cuda):
    import torch

    from zillumgl_gb300.scene import DiffRenderer, Scene

    data = diff_scene(seed=11, width=512, height=512)
    assert data.materials.size // 16 >= 8
    spp, params = 32, dict(max_depth=6)
    sc = Scene(data)
    dr = DiffRenderer(sc, spp, **params)
    img = dr.forward().cpu().numpy().reshape(-1, 3)
    rng = np.random.default_rng(44)
    pix = np.sort(rng.choice(512 * 512, 2048, replace=False)).astype(np.int32)
    orc = oracle.OracleScene(data, sc.export("sobol"), params)
    ref_img = orc.render_pt(pix, spp) / np.float32(spp)
    assert _same_bits(img[pix], ref_img), "forward image differs from the oracle on the sampled pixels"
    dimage = np.zeros((512 * 512, 3), np.float32)
    dimage[pix] = rng.uniform(-1.0, 1.0, (pix.size, 3)).astype(np.float32)
    dimage = dimage.reshape(512, 512, 3)
    g = dr.backward(torch.from_numpy(dimage).to(cuda)).cpu().numpy().astype(np.float64)
    ref = orc.diff_grad(data, spp, dimage)
    assert g.shape == ref.shape == (51,)
    err = np.abs(g - ref)
    tol = GRAD_ABS * np.abs(ref).max() + GRAD_REL * np.abs(ref)
    worst = int(np.argmax(err / tol))
    assert np.all(err <= tol), f"param {worst}: gpu {g[worst]:.6g} oracle {ref[worst]:.6g}"
    dr.close()
    sc.close()
