"""Batched wavefront renderer vs the plain path integrator.

Each request's frame after one zgl_batch_render must equal, bit for bit, the
frame of a fresh ZGL_INTEGRATOR_PATH integrator after `spp` passes: the
batched schedule changes which lane renders which sample and when, not the
arithmetic, the RNG streams or the per-pixel summation order.  Checked for
uneven requests (scenes, film sizes, spp, depth, Russian roulette, sampler),
for every schedule (flat, persistent, shared-memory queues) and several
settings (block size, queue capacity, regeneration threshold)
and after autotuning and graph replay.
"""
from __future__ import annotations

import numpy as np
import pytest

from zillumgl_gb300.scene import BatchRenderer, PathIntegrator, Scene, default_params
from zillumgl_gb300.synthetic import cornell_scene, sky_environment

pytestmark = pytest.mark.gpu


def _requests(cuda):
    import torch

    specs = [
        (cornell_scene(seed=21, width=40, height=24), 5, dict(max_depth=5)),
        (cornell_scene(seed=22, width=17, height=31, sampler=0), 3, dict(max_depth=3)),
        (cornell_scene(seed=23, width=33, height=33), 7, dict(max_depth=8, russian_roulette=1, rr_start_depth=3)),
        (cornell_scene(seed=24, width=8, height=8), 1, dict(max_depth=4)),
    ]
    d = cornell_scene(seed=25, width=24, height=20)
    d.env_rgb = sky_environment(32, 16, seed=6)
    specs.append((d.normalized(), 4, dict(max_depth=4, light_env_uniform_sample=1, light_portion=0.4)))
    out = []
    for data, spp, params in specs:
        sc = Scene(data)
        W, H = data.film
        frame = torch.full((H, W, 4), 7.0, dtype=torch.float32, device=cuda)
        out.append((sc, spp, params, frame))
    return out


def _plain(sc, spp, params):
    integ = PathIntegrator(sc, **params)
    for _ in range(spp):
        integ.render_one_pass()
    f, n = integ.get_frame()
    integ.close()
    return f


@pytest.fixture(scope="module")
def batch_setup(zgl_lib, cuda):
    reqs = _requests(cuda)
    refs = [_plain(sc, spp, params) for sc, spp, params, _ in reqs]
    yield reqs, refs
    for sc, *_ in reqs:
        sc.close()


def _check(reqs, refs):
    import torch

    torch.cuda.synchronize()
    for i, ((_, _, _, frame), ref) in enumerate(zip(reqs, refs)):
        got = frame.cpu().numpy()
        bad = np.sum(np.any(got.view(np.uint32) != ref.view(np.uint32), axis=-1))
        assert bad == 0, f"request {i}: {bad} pixels differ from the plain integrator"


FLAT, PERSISTENT, QUEUE = 1, 2, 3


@pytest.mark.parametrize("cfg", [
    dict(),
    dict(schedule=FLAT),
    dict(schedule=PERSISTENT),
    dict(schedule=PERSISTENT, block_size=64, queue_capacity=8, regen_threshold=1),
    dict(schedule=PERSISTENT, block_size=256, queue_capacity=128, regen_threshold=32),
    dict(schedule=PERSISTENT, block_size=128, queue_capacity=1, regen_threshold=8),
    dict(schedule=FLAT, scratch_mib=1),        # chunks of a few sample indices
    dict(schedule=PERSISTENT, scratch_mib=1),
    dict(schedule=QUEUE),
    dict(schedule=QUEUE, block_size=256, queue_capacity=1, regen_threshold=1),
    dict(schedule=QUEUE, block_size=256, queue_capacity=128, regen_threshold=32),
    dict(schedule=QUEUE, scratch_mib=1),
])
def test_batch_equals_plain_integrator(batch_setup, cfg):
    reqs, refs = batch_setup
    b = BatchRenderer(reqs, **cfg)
    b.render()
    _check(reqs, refs)
    # replaying the captured graph gives the same frames again
    b.render()
    _check(reqs, refs)
    b.close()


def test_autotune_then_render(batch_setup):
    reqs, refs = batch_setup
    b = BatchRenderer(reqs)
    chosen = b.autotune()
    assert chosen["schedule"] in (FLAT, PERSISTENT, QUEUE)
    assert chosen["block_size"] in (64, 128, 256)
    assert b.config() == chosen
    b.render()
    _check(reqs, refs)
    b.close()


def test_autotune_cache_reuses_the_choice(batch_setup, tmp_path):
    import json

    reqs, refs = batch_setup
    path = tmp_path / "tune.json"
    b = BatchRenderer(reqs)
    first = b.autotune(cache=path)
    b.close()
    table = json.loads(path.read_text())
    assert list(table.values()) == [first]
    b2 = BatchRenderer(reqs)
    assert b2.autotune(cache=path) == first  # from the file, untimed
    assert b2.config() == first
    b2.render()
    _check(reqs, refs)
    b2.close()


@pytest.mark.parametrize("schedule", [FLAT, PERSISTENT, QUEUE])
def test_batch_in_sample_chunks(zgl_lib, cuda, schedule):
    """A 1 MiB scratch budget forces one sample index per launch for a 256^2
    request; frames still equal the plain integrator's bit for bit."""
    import torch

    specs = [(cornell_scene(seed=31, width=256, height=256), 6, dict(max_depth=4)),
             (cornell_scene(seed=32, width=24, height=16), 3, dict(max_depth=5))]
    reqs = []
    for data, spp, params in specs:
        sc = Scene(data)
        W, H = data.film
        reqs.append((sc, spp, params, torch.zeros((H, W, 4), dtype=torch.float32, device=cuda)))
    refs = [_plain(sc, spp, params) for sc, spp, params, _ in reqs]
    b = BatchRenderer(reqs, schedule=schedule, scratch_mib=1)
    b.render()
    _check(reqs, refs)
    b.close()
    for sc, *_ in reqs:
        sc.close()


def test_batch_and_multipass_argument_errors(zgl_lib, cuda):
    import torch

    from zillumgl_gb300 import ZglError
    from zillumgl_gb300.scene import PathIntegrator

    sc = Scene(cornell_scene(seed=33, width=8, height=8))
    frame = torch.zeros((8, 8, 4), dtype=torch.float32, device=cuda)
    for bad in (dict(schedule=7), dict(scratch_mib=-1), dict(schedule=PERSISTENT, block_size=96),
                dict(schedule=PERSISTENT, regen_threshold=33)):
        with pytest.raises(ZglError):
            BatchRenderer([(sc, 2, dict(max_depth=3), frame)], **bad)
    with pytest.raises(ZglError):
        BatchRenderer([(sc, 0, dict(max_depth=3), frame)])
    it = PathIntegrator(sc, max_depth=3)
    with pytest.raises(ZglError):
        it.render_passes(-1)
    it.render_passes(0)  # no-op
    _, spp = it.get_frame()
    assert spp == 0
    it.close()
    sc.close()
