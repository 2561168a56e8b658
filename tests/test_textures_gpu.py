"""Albedo textures (material_loader.glsl:8-79, Texture.cpp:134-171) in every
integrator against the oracle: the path tracer bit for bit on textured
Lambertian, principled, metal-workflow and dielectric surfaces, the light
tracer and triple integrator within the 1e-4 relative film tolerance, the
batched renderer bit-identical to the plain integrator, and the adjoint
within its gradient tolerance (a textured triangle's base colour is the
texture's, so its material's baseColor gets no gradient from it)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300.scene import (BatchRenderer, DiffRenderer, LightIntegrator, PathIntegrator, Scene,
                                  TripleIntegrator)
from zillumgl_gb300.synthetic import textured_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("base,params", [
    ("cornell", dict(max_depth=5)),
    ("zoo", dict(max_depth=8)),
    ("zoo", dict(max_depth=10, russian_roulette=1, rr_start_depth=3)),
])
def test_path_tracer_bit_exact_with_textures(zgl_lib, cuda, base, params):
    d = textured_scene(seed=52, width=48, height=40, base=base)
    sc = Scene(d)
    integ = PathIntegrator(sc, **params)
    for _ in range(3):
        integ.render_one_pass()
    frame, _ = integ.get_frame()
    W, H = d.film
    ref = oracle.OracleScene(d, sc.export("sobol"), params).render_pt(np.arange(W * H), 3).reshape(H, W, 3)
    got = frame[..., :3]
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), \
        f"{int(np.sum(np.any(got != ref, axis=-1)))} pixels differ"
    # the textures change the image: the untextured scene renders differently
    plain = textured_scene(seed=52, width=48, height=40, base=base)
    plain.obj_mat_tex = plain.obj_mat_tex | np.int32(-65536)
    ref_plain = oracle.OracleScene(plain, sc.export("sobol"), params).render_pt(np.arange(W * H), 3)
    assert np.abs(ref_plain.reshape(H, W, 3) - ref).max() > 0.05
    integ.close()
    sc.close()


def _film_close(got, ref):
    from tests.test_light_gpu import _check

    _check(got, ref)


def test_light_tracer_with_textures(zgl_lib, cuda):
    d = textured_scene(seed=53, width=40, height=32, base="zoo")
    sc = Scene(d)
    params = dict(max_depth=8, blocks_per_pass=8)
    integ = LightIntegrator(sc, **params)
    for _ in range(2):
        integ.render_one_pass()
    frame, _ = integ.get_frame()
    ref = oracle.OracleScene(d, sc.export("sobol"), params).render_lt(2, blocks=8)
    _film_close(frame[..., :3], ref)
    assert ref.sum() > 0
    integ.close()
    sc.close()


def test_triple_integrator_with_textures(zgl_lib, cuda):
    d = textured_scene(seed=54, width=32, height=24)
    sc = Scene(d)
    params = dict(max_depth=8, blocks_per_pass=16, loops_per_pass=1)
    integ = TripleIntegrator(sc, **params)
    for _ in range(2):
        integ.render_one_pass()
    frame, _ = integ.get_frame()
    ref = oracle.OracleScene(d, sc.export("sobol"), params).render_triple(2, blocks=16, loops=1)
    _film_close(frame[..., :3], ref)
    integ.close()
    sc.close()


def test_batched_renderer_with_textures(zgl_lib, cuda):
    import torch

    d = textured_scene(seed=55, width=40, height=24, base="zoo")
    sc = Scene(d)
    params = dict(max_depth=6)
    plain = PathIntegrator(sc, **params)
    plain.render_passes(3)
    ref, _ = plain.get_frame()
    plain.close()
    for schedule in (1, 2):  # ZGL_BATCH_FLAT, ZGL_BATCH_PERSISTENT
        frame = torch.zeros((24, 40, 4), dtype=torch.float32, device=cuda)
        b = BatchRenderer([(sc, 3, params, frame)], schedule=schedule)
        b.render()
        torch.cuda.synchronize()
        assert np.array_equal(frame.cpu().numpy().view(np.uint32), ref.view(np.uint32)), schedule
        b.close()
    sc.close()


def test_adjoint_with_textures(zgl_lib, cuda):
    import torch

    d = textured_scene(seed=56, width=32, height=24, base="diff")
    params = dict(max_depth=6)
    sc = Scene(d)
    dr = DiffRenderer(sc, 2, **params)
    dr.forward()
    dimg = np.random.default_rng(6).uniform(-1, 1, (24, 32, 3)).astype(np.float32)
    g = dr.backward(torch.from_numpy(dimg).cuda()).cpu().numpy().astype(np.float64)
    ref = oracle.OracleScene(d, sc.export("sobol"), params).diff_grad(d, 2, dimg)
    err = np.abs(g - ref)
    tol = 2e-3 * np.abs(ref).max() + 1e-3 * np.abs(ref)
    worst = int(np.argmax(err / tol))
    assert np.all(err <= tol), f"param {worst}: gpu {g[worst]:.6g} oracle {ref[worst]:.6g}"
    # the floor (material 0) is textured everywhere: no baseColor gradient
    assert np.all(g[0:3] == 0.0) and np.all(ref[0:3] == 0.0)
    assert np.abs(g[3:6]).max() > 0  # its roughness, metallic and specular still get one
    dr.close()
    sc.close()
