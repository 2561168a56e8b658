"""The FP64 gradient oracle of the differentiable renderer against central
finite differences of the oracle's own forward render (common random numbers:
every sample reuses its seeds).

Plain finite differences only check parameters that leave every sampling
decision unchanged: baseColor and specular (no pdf depends on them) and light
power (with one light and no environment the selection probabilities do not
change).  Roughness and metallic also steer the GGX sample and the lobe
choice, so they are checked against finite differences of the frozen-sampling
estimator (OracleScene.render_pt_frozen): every direction, lobe pick, pdf, MIS
weight and Russian-roulette decision is the one taken at the unperturbed
parameters and only the BSDF values move, which is the estimator the
detached-sampling adjoint differentiates.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300.synthetic import diff_scene

SPP = 2
PARAMS = dict(max_depth=3)
H_FD = 1e-3


@pytest.fixture(scope="module")
def setup():
    from zillumgl_gb300.scene import Scene

    d = diff_scene(seed=21, width=12, height=10)
    sobol = Scene(d, host_only=True).export("sobol")
    rng = np.random.default_rng(4)
    W, H = d.film
    dimage = rng.uniform(-1.0, 1.0, (H, W, 3)).astype(np.float32)
    return d, sobol, dimage


def _loss(d, sobol, dimage):
    W, H = d.film
    orc = oracle.OracleScene(d, sobol, PARAMS)
    img = orc.render_pt(np.arange(W * H), SPP, spp0=0, fc0=1).astype(np.float64) / SPP
    return float(np.sum(img.reshape(H, W, 3) * dimage))


def _perturbed(d, slot, h):
    e = type(d)(**{k: (np.array(v, copy=True) if isinstance(v, np.ndarray) else v) for k, v in vars(d).items()})
    nmat = d.materials.shape[0]
    if slot < 6 * nmat:
        m, i = divmod(slot, 6)
        col = [0, 1, 2, 3, 5, 6][i]
        e.materials[m, col] += np.float32(h)
    else:
        k, c = divmod(slot - 6 * nmat, 3)
        e.light_power[k, c] += np.float32(h)
    return e


def test_oracle_gradient_matches_central_differences(setup):
    d, sobol, dimage = setup
    orc = oracle.OracleScene(d, sobol, PARAMS)
    g = orc.diff_grad(d, SPP, dimage, nthreads=4)
    nmat = d.materials.shape[0]
    assert g.shape == (6 * nmat + 3,)
    # baseColor of materials 0, 5 (the boxes) and 6 (the sphere), specular of
    # material 2, and the light power
    slots = [0, 1, 2, 30, 31, 32, 36, 38, 6 * 2 + 5, 6 * nmat, 6 * nmat + 1, 6 * nmat + 2]
    for slot in slots:
        base = d.materials[slot // 6, [0, 1, 2, 3, 5, 6][slot % 6]] if slot < 6 * nmat else 15.0
        h = H_FD * max(1.0, abs(float(base)))
        fd = (_loss(_perturbed(d, slot, h), sobol, dimage) - _loss(_perturbed(d, slot, -h), sobol, dimage)) / (2 * h)
        scale = max(abs(fd), 1e-3 * np.abs(g).max())
        assert abs(g[slot] - fd) <= 2e-3 * scale, f"slot {slot}: oracle {g[slot]:.6g} fd {fd:.6g}"


def test_oracle_gradient_is_linear_in_the_image_adjoint(setup):
    d, sobol, dimage = setup
    orc = oracle.OracleScene(d, sobol, PARAMS)
    g1 = orc.diff_grad(d, SPP, dimage, nthreads=4)
    g2 = orc.diff_grad(d, SPP, 4.0 * dimage, nthreads=4)
    np.testing.assert_allclose(g2, 4.0 * g1, rtol=1e-12, atol=1e-15)
    assert np.abs(g1).max() > 0


def _frozen_loss(orc, d, materials, dimage):
    W, H = d.film
    img = orc.render_pt_frozen(materials, np.arange(W * H), SPP).astype(np.float64) / SPP
    return float(np.sum(img.reshape(H, W, 3) * dimage))


def test_oracle_gradient_matches_frozen_sampling_differences(setup):
    """Roughness (raw, before the 0.0134 remap of material_loader.glsl:46) and
    metallic (which also drives the lobe pick of material.glsl:537-540) of
    every principled material, and baseColor / specular as a cross-check."""
    d, sobol, dimage = setup
    orc = oracle.OracleScene(d, sobol, PARAMS)
    g = orc.diff_grad(d, SPP, dimage, nthreads=4)
    nmat = d.materials.shape[0]
    slots = [6 * m + 3 for m in range(nmat)] + [6 * m + 4 for m in range(nmat)] + [0, 6 * 2 + 5]
    checked = 0
    for slot in slots:
        m, i = divmod(slot, 6)
        col = [0, 1, 2, 3, 5, 6][i]
        base = float(d.materials[m, col])
        h = H_FD * max(1.0, abs(base))
        mp, mm = d.materials.copy(), d.materials.copy()
        mp[m, col] += np.float32(h)
        mm[m, col] -= np.float32(h)
        hh = (float(mp[m, col]) - float(mm[m, col])) / 2
        fd = (_frozen_loss(orc, d, mp, dimage) - _frozen_loss(orc, d, mm, dimage)) / (2 * hh)
        scale = max(abs(fd), 1e-3 * np.abs(g).max())
        assert abs(g[slot] - fd) <= 5e-3 * scale, f"slot {slot}: oracle {g[slot]:.6g} fd {fd:.6g}"
        checked += abs(fd) > 1e-3 * np.abs(g).max()
    assert checked >= nmat  # most of the roughness / metallic derivatives are not negligible
