"""The CUDA path against outputs of the reference's own code.

tests/golden/reference_pins.json holds outputs of the reference's
BVH::build() (src/accelerator/BVH.cpp compiled unchanged) and of its
path_integ_naive / light_path_integ / triple_path_pass_{pt,lpt} compute
shaders and bvhHit / bvhTest (compiled as C++ by oracle/glsl_to_cpp.py),
made by tests/golden/make_reference_pins.py where the reference tree is
present.  Here, on the GPU, through the C ABI:

* path-tracer frames hash to the reference shader's frames (bit for bit);
* light-tracer and triple-integrator films agree within 1e-4 per pixel (the
  GPU splats with float atomics, so the summation order differs);
* the device-built PackedBVH of the 1M soup hashes to BVH::build()'s;
* closest-hit and any-hit results on a 60k soup with mixed rays hash to the
  reference shader's.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from tests.golden.make_reference_pins import decode
from tests.reference_pin_cases import FILM_CASES, FRAME_CASES, SOUPS, TRACE_CASE, frame_rgb, mixed_rays, sha256
from zillumgl_gb300 import BVH
from zillumgl_gb300.synthetic import TRAVERSAL_SEEDS, triangle_soup

pytestmark = pytest.mark.gpu

PINS = json.loads((Path(__file__).resolve().parent / "golden" / "reference_pins.json").read_text())


@pytest.mark.parametrize("name", list(FRAME_CASES))
def test_path_tracer_frame_equals_reference_shader(zgl_lib, cuda, name):
    from zillumgl_gb300.scene import PathIntegrator, Scene

    make, params, passes = FRAME_CASES[name]
    d = make()
    sc = Scene(d)
    integ = PathIntegrator(sc, **params)
    for _ in range(passes):
        integ.render_one_pass()
    frame, spp = integ.get_frame()
    integ.close()
    sc.close()
    pin = PINS["frames"][name]
    assert spp == passes and list(d.film) == pin["film"]
    rgb = frame_rgb(frame)
    assert sha256(rgb) == pin["sha256"], f"{name}: frame differs from the reference shader's (mean {rgb.mean():.6g} " \
                                         f"vs {pin['mean']:.6g})"


@pytest.mark.parametrize("name", list(FILM_CASES))
def test_light_and_triple_films_match_reference_shaders(zgl_lib, cuda, name):
    from zillumgl_gb300.scene import LightIntegrator, Scene, TripleIntegrator

    kind, make, params, passes, blocks, loops = FILM_CASES[name]
    d = make()
    sc = Scene(d)
    if kind == "light":
        integ = LightIntegrator(sc, **params, blocks_per_pass=blocks)
    else:
        integ = TripleIntegrator(sc, **params, blocks_per_pass=blocks, loops_per_pass=loops)
    for _ in range(passes):
        integ.render_one_pass()
    frame, _ = integ.get_frame()
    integ.close()
    sc.close()
    pin = PINS["films"][name]
    ref = decode(pin["film"], pin["shape"])
    got = frame_rgb(frame)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-5)
    assert rel.max() <= 1e-4, f"{name}: max rel {rel.max():.3g}"
    assert ref.sum() > 0


def test_device_build_equals_reference_builder(zgl_lib, cuda):
    n = SOUPS["soup_1M"]
    v, idx = triangle_soup(n, TRAVERSAL_SEEDS[n])
    acc = BVH(v, idx).build_device()
    p = acc.export()
    acc.close()
    assert sha256(p.bounds, p.hitTable) == PINS["soups"]["soup_1M"]["sha256"]


def test_traversal_equals_reference_shader(zgl_lib, cuda):
    import torch

    name, ntri, seed, nray, rseed = TRACE_CASE
    pin = PINS["trace"][name]
    v, idx = triangle_soup(ntri, seed)
    acc = BVH(v, idx).build()
    p = acc.export()
    assert sha256(p.bounds, p.hitTable) == pin["bvh_sha256"]
    o, d = mixed_rays(np.random.default_rng(rseed), nray)
    to, td = torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda)
    for schedule in ("auto", "thread_per_ray", "persistent", "prefetch"):
        acc.set_trace_schedule(schedule)
        hid, ht = acc.trace_closest(to, td)
        torch.cuda.synchronize()
        assert sha256(hid.cpu().numpy(), ht.cpu().numpy()) == pin["closest_sha256"], schedule
        tmax = torch.from_numpy(np.random.default_rng(rseed + 1).random(nray).astype(np.float32)).to(cuda)
        occ = acc.trace_any(to, td, tmax).cpu().numpy().astype(np.int32)
        assert sha256(occ) == pin["any_sha256"], schedule
    acc.close()
