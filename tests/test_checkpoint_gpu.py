"""Checkpoint / resume of the integrators (zgl_integrator_save/restore; the
reference's Scene::saveToFile is empty, Scene.cpp:129-131).  The samplers are
counter-based, so a path tracer restored from a checkpoint continues bit for
bit like one that never stopped; the light and triple integrators splat with
float atomics, so they agree to float-summation order."""
from __future__ import annotations

import numpy as np
import pytest

from zillumgl_gb300 import ZglError
from zillumgl_gb300.scene import LightIntegrator, PathIntegrator, Scene, TripleIntegrator
from zillumgl_gb300.synthetic import cornell_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cls,params", [
    (PathIntegrator, dict(max_depth=5, russian_roulette=1, rr_start_depth=2)),
    (LightIntegrator, dict(max_depth=5, blocks_per_pass=8)),
    (TripleIntegrator, dict(max_depth=5, blocks_per_pass=8, loops_per_pass=1)),
])
def test_resume_continues_like_an_uninterrupted_render(zgl_lib, cuda, cls, params):
    d = cornell_scene(seed=61, width=40, height=32, sampler=0 if cls is not PathIntegrator else 1)
    sc = Scene(d)
    straight = cls(sc, **params)
    for _ in range(5):
        straight.render_one_pass()
    ref, spp_ref = straight.get_frame()
    scale_ref = straight.result_scale()

    first = cls(sc, **params)
    for _ in range(3):
        first.render_one_pass()
    state, total = first.save()
    first.close()
    assert state["cur_sample"] == 3
    resumed = cls(sc, **params)
    resumed.restore(state, total)
    for _ in range(2):
        resumed.render_one_pass()
    got, spp = resumed.get_frame()
    assert spp == spp_ref and resumed.result_scale() == scale_ref
    if cls is PathIntegrator:
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    else:
        assert np.allclose(got, ref, rtol=1e-5, atol=1e-6)
    # a checkpoint only restores into an integrator of the same kind
    # (light and triple films have the same size: the kind check rejects them)
    other = {PathIntegrator: LightIntegrator, LightIntegrator: TripleIntegrator,
             TripleIntegrator: LightIntegrator}[cls](sc, max_depth=5)
    with pytest.raises((ZglError, ValueError)):
        other.restore(state, total)
    for x in (straight, resumed, other):
        x.close()
    sc.close()
