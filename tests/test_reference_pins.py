"""The oracle against the reference's own code, on the CPU.

* MTBVH build: the reference's BVH::build() (src/accelerator/BVH.cpp:116-345
  and AABB.cpp, compiled unchanged from the reference tree behind stand-in
  glm / OpenGL headers) gives the same PackedBVH as the oracle restatement and
  the product's host builder, bit for bit, on every host-builder case
  (soups, a shared-vertex grid, identical and collinear centroids, 1-5
  triangles, signed zeros).
* Shaders: the reference's path_integ_naive.glsl, light_path_integ.glsl and
  triple_path_pass_{pt,lpt}.glsl, turned into C++ by the mechanical
  transform of oracle/glsl_to_cpp.py, give the same frames and films as the
  oracle restatement bit for bit; their bvhHit / bvhTest give the same hits.
* The fixture tests/golden/reference_pins.json, which the GPU tests read on
  machines without the reference tree, still matches the reference code.

Every test here is skipped where the reference tree is absent.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from tests.reference_pin_cases import FILM_CASES, FRAME_CASES, SOUPS, TRACE_CASE, frame_rgb, mixed_rays, sha256
from tests.test_bvh_host import _cases
from zillumgl_gb300.scene import Scene
from zillumgl_gb300.synthetic import TRAVERSAL_SEEDS, primary_rays, shadow_tmax, triangle_soup

PINS = json.loads((Path(__file__).resolve().parent / "golden" / "reference_pins.json").read_text())


@pytest.fixture(scope="module")
def ref():
    if oracle.ref_lib() is None:
        pytest.skip("reference tree not present")


@pytest.fixture(scope="module")
def glsl():
    if oracle.glsl_lib() is None:
        pytest.skip("reference tree not present")


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name,v,idx", list(_cases()), ids=lambda x: x if isinstance(x, str) else "")
def test_reference_builder_equals_oracle_and_host_builder(ref, zgl_lib, name, v, idx):
    from zillumgl_gb300 import BVH

    rb, rh = oracle.ref_bvh_build(v, idx)
    ob, oh, _ = oracle.bvh_build(v, idx)
    assert np.array_equal(_bits(rb), _bits(ob)), f"{name}: oracle bounds differ from BVH::build()"
    assert np.array_equal(rh, oh), f"{name}: oracle hit tables differ from BVH::build()"
    pb = BVH(v, idx).build_host()
    assert np.array_equal(_bits(pb.bounds), _bits(rb)) and np.array_equal(pb.hitTable, rh), name


def test_reference_builder_1M_soup_matches_fixture(ref):
    n = SOUPS["soup_1M"]
    v, idx = triangle_soup(n, TRAVERSAL_SEEDS[n])
    rb, rh = oracle.ref_bvh_build(v, idx)
    assert sha256(rb, rh) == PINS["soups"]["soup_1M"]["sha256"]
    ob, oh, _ = oracle.bvh_build(v, idx)
    assert np.array_equal(_bits(rb), _bits(ob)) and np.array_equal(rh, oh)


def test_reference_shader_traversal_equals_oracle(ref, glsl):
    name, ntri, seed, nray, rseed = TRACE_CASE
    v, idx = triangle_soup(ntri, seed)
    b, h = oracle.ref_bvh_build(v, idx)
    o, d = mixed_rays(np.random.default_rng(rseed), nray)
    gh, gt = oracle.glsl_trace(b, h, v, idx, o, d)
    oh, ot, _, _ = oracle.trace(b, h, v, idx, o, d)
    assert np.array_equal(gh, oh) and np.array_equal(_bits(gt), _bits(ot))
    tmax = np.random.default_rng(rseed + 1).random(nray).astype(np.float32)
    ga, _ = oracle.glsl_trace(b, h, v, idx, o, d, tmax=tmax)
    oa, _, _, _ = oracle.trace(b, h, v, idx, o, d, tmax=tmax, any_hit=True)
    assert np.array_equal(ga, oa)
    pin = PINS["trace"][name]
    assert sha256(b, h) == pin["bvh_sha256"]
    assert sha256(gh, gt) == pin["closest_sha256"] and sha256(ga) == pin["any_sha256"]
    # coherent rays too
    op, dp = primary_rays(128, 128)
    gh, gt = oracle.glsl_trace(b, h, v, idx, op, dp)
    oh, ot, _, _ = oracle.trace(b, h, v, idx, op, dp)
    assert np.array_equal(gh, oh) and np.array_equal(_bits(gt), _bits(ot))
    tm = 1.0 + shadow_tmax(op.shape[0], 9)
    ga, _ = oracle.glsl_trace(b, h, v, idx, op, dp, tmax=tm)
    oa, _, _, _ = oracle.trace(b, h, v, idx, op, dp, tmax=tm, any_hit=True)
    assert np.array_equal(ga, oa)


@pytest.mark.parametrize("name", list(FRAME_CASES))
def test_reference_path_tracer_shader_equals_oracle(glsl, name):
    make, params, passes = FRAME_CASES[name]
    d = make()
    sc = Scene(d, host_only=True)
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    W, H = d.film
    pix = np.arange(W * H)
    g = orc.glsl_render_pt(pix, passes)
    o = orc.render_pt(pix, passes)
    sc.close()
    bad = np.nonzero(np.any(_bits(g) != _bits(o), axis=1))[0]
    assert bad.size == 0, f"{bad.size} pixels differ from the reference shader, first {bad[:5]}"
    assert sha256(frame_rgb(g.reshape(H, W, 3))) == PINS["frames"][name]["sha256"]
    assert o.mean() > 0


@pytest.mark.parametrize("name", list(FILM_CASES))
def test_reference_light_and_triple_shaders_equal_oracle(glsl, name):
    kind, make, params, passes, blocks, loops = FILM_CASES[name]
    d = make()
    sc = Scene(d, host_only=True)
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    if kind == "light":
        g, o = orc.glsl_render_lt(passes, blocks=blocks), orc.render_lt(passes, blocks=blocks)
    else:
        g = orc.glsl_render_triple(passes, blocks=blocks, loops=loops)
        o = orc.render_triple(passes, blocks=blocks, loops=loops)
    sc.close()
    assert np.array_equal(_bits(g), _bits(o)), f"{name}: film differs from the reference shaders"
    from tests.golden.make_reference_pins import decode

    pin = PINS["films"][name]
    assert np.array_equal(_bits(decode(pin["film"], pin["shape"])), _bits(g))
    assert o.sum() > 0
