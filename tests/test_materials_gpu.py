"""Metal-workflow, dielectric (smooth and rough) and thin-dielectric BSDFs
(material.glsl:85-355) in every integrator against the oracle: the path
tracer bit for bit, the light tracer and triple integrator within the 1e-4
relative film tolerance (float atomics), the adjoint within its gradient
tolerance (those materials carry no differentiable parameter)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300.scene import DiffRenderer, LightIntegrator, PathIntegrator, Scene, TripleIntegrator
from zillumgl_gb300.synthetic import material_zoo_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("params", [dict(max_depth=8), dict(max_depth=10, russian_roulette=1, rr_start_depth=3)])
def test_path_tracer_bit_exact_with_every_material(zgl_lib, cuda, params):
    d = material_zoo_scene(seed=41, width=48, height=40)
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
    assert ref.mean() > 0.02
    integ.close()
    sc.close()


def _film_close(got, ref):
    from tests.test_light_gpu import _check

    _check(got, ref)


def test_light_tracer_with_every_material(zgl_lib, cuda):
    d = material_zoo_scene(seed=42, width=40, height=32)
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


def test_triple_integrator_with_every_material(zgl_lib, cuda):
    d = material_zoo_scene(seed=43, width=32, height=24)
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


def test_adjoint_with_every_material(zgl_lib, cuda):
    import torch

    d = material_zoo_scene(seed=44, width=32, height=24)
    params = dict(max_depth=8)
    sc = Scene(d)
    dr = DiffRenderer(sc, 2, **params)
    dr.forward()
    dimg = np.random.default_rng(5).uniform(-1, 1, (24, 32, 3)).astype(np.float32)
    g = dr.backward(torch.from_numpy(dimg).cuda()).cpu().numpy().astype(np.float64)
    ref = oracle.OracleScene(d, sc.export("sobol"), params).diff_grad(d, 2, dimg)
    err = np.abs(g - ref)
    assert np.all(err <= 2e-3 * np.abs(ref).max() + 1e-3 * np.abs(ref))
    assert np.all(g[5 * 6:9 * 6] == 0.0) and np.all(ref[5 * 6:9 * 6] == 0.0)  # materials 5-8 not differentiable
    dr.close()
    sc.close()
