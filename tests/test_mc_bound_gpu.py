"""Monte Carlo accuracy of the GPU path tracer against a 4096-spp oracle image.

The GPU renders N = 64 samples per pixel; the oracle renders 4096 further
samples (sample indices 64..4159, so the two estimates share no sample).
Per pixel, z = |mean_gpu - mean_ref| / sqrt(s^2 / N + s^2 / 4096) with s the
standard deviation of the GPU's 64 per-sample values.  The bound: at least
97% of the pixels with s > 0 have z <= 3 (a Gaussian gives 99.7%; the
per-sample radiance has heavy tails at 64 spp), pixels with s = 0 agree to
1e-4 relative, and the image means agree within 3 standard errors.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300.scene import PathIntegrator, Scene
from zillumgl_gb300.synthetic import cornell_scene

pytestmark = pytest.mark.gpu

N_GPU = 64
N_REF = 4096


def _per_sample_frames(sc, params, n):
    integ = PathIntegrator(sc, **params)
    prev = None
    out = []
    for _ in range(n):
        integ.render_one_pass()
        frame, _ = integ.get_frame()
        cur = frame[..., :3].astype(np.float64)
        out.append(cur if prev is None else cur - prev)
        prev = cur
    integ.close()
    return np.stack(out)


@pytest.mark.parametrize("case", ["cornell", "env_two_lights"])
def test_three_sigma_bound_against_4096_spp_oracle(zgl_lib, cuda, case):
    if case == "cornell":
        d, params = cornell_scene(seed=1, width=32, height=32), dict(max_depth=5)
    else:
        from tests.test_tables import _multi_light_scene

        d, params = _multi_light_scene(env=True, w=32, h=24), dict(max_depth=4)
    sc = Scene(d)
    samples = _per_sample_frames(sc, params, N_GPU)
    W, H = d.film
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    ref = orc.render_pt(np.arange(W * H), N_REF, spp0=N_GPU, fc0=N_GPU + 1).reshape(H, W, 3).astype(np.float64)
    ref /= N_REF
    sc.close()
    mean = samples.mean(axis=0)
    s = samples.std(axis=0, ddof=1)
    se = s * np.sqrt(1.0 / N_GPU + 1.0 / N_REF)
    noisy = s > 0
    z = np.abs(mean - ref)[noisy] / se[noisy]
    frac = float(np.mean(z <= 3.0))
    assert frac >= 0.97, f"only {frac:.4f} of the noisy pixel channels within 3 sigma"
    flat = ~noisy
    if flat.any():
        np.testing.assert_allclose(mean[flat], ref[flat], rtol=1e-4, atol=1e-6)
    img_se = samples.mean(axis=(1, 2, 3)).std(ddof=1) * np.sqrt(1.0 / N_GPU + 1.0 / N_REF)
    assert abs(mean.mean() - ref.mean()) <= 3.0 * img_se + 1e-7
    assert ref.mean() > 0.01
