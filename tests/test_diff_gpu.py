"""Differentiable path tracer on the GPU (zgl_diff_*).

* forward: the image is the mean of the path tracer's first spp samples,
  bit-identical to the oracle's render and to the progressive integrator;
* backward: the path-replay gradient against the oracle's FP64 adjoint
  (every parameter, including roughness and metallic) and against central
  finite differences of the GPU forward with common random numbers (the
  parameters no sampling decision depends on);
* a torch.autograd.Function around forward/backward (test harness only)
  driving a few steps of inverse rendering.

Gradient tolerance: per parameter |gpu - oracle| <= 2e-3 * max(|oracle|) +
1e-3 * |oracle| (float32 accumulation with atomics against FP64).
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import ZglError
from zillumgl_gb300.scene import DiffRenderer, PathIntegrator, Scene
from zillumgl_gb300.synthetic import cornell_scene, diff_scene

pytestmark = pytest.mark.gpu

GRAD_ABS = 2e-3
GRAD_REL = 1e-3


def _setup(d, spp, params, seed=4):
    import torch

    sc = Scene(d)
    dr = DiffRenderer(sc, spp, **params)
    W, H = d.film
    rng = np.random.default_rng(seed)
    dimage = rng.uniform(-1.0, 1.0, (H, W, 3)).astype(np.float32)
    return sc, dr, dimage, torch.from_numpy(dimage).cuda()


def test_forward_is_the_sample_mean_bit_exact(zgl_lib, cuda):
    d = diff_scene(seed=21, width=40, height=24)
    params = dict(max_depth=5)
    sc, dr, _, _ = _setup(d, 3, params)
    img = dr.forward().cpu().numpy()
    W, H = d.film
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    ref = (orc.render_pt(np.arange(W * H), 3, spp0=0, fc0=1) / np.float32(3)).reshape(H, W, 3)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    integ = PathIntegrator(sc, **params)
    for _ in range(3):
        integ.render_one_pass()
    frame, _ = integ.get_frame()
    assert np.array_equal(img.view(np.uint32), (frame[..., :3] / np.float32(3)).view(np.uint32))
    assert img.mean() > 0.02


@pytest.mark.parametrize("case", ["principled", "cornell_rr", "env_two_lights"])
def test_backward_matches_fp64_oracle_adjoint(zgl_lib, cuda, case):
    if case == "principled":
        d, spp, params = diff_scene(seed=22, width=32, height=24), 2, dict(max_depth=6)
    elif case == "cornell_rr":
        d, spp, params = cornell_scene(seed=23, width=24, height=24), 2, dict(max_depth=6, russian_roulette=1,
                                                                              rr_start_depth=2)
    else:
        from tests.test_tables import _multi_light_scene

        d, spp, params = _multi_light_scene(env=True, w=24, h=16), 2, dict(max_depth=4)
    sc, dr, dimage, dimg_t = _setup(d, spp, params)
    dr.forward()
    g = dr.backward(dimg_t).cpu().numpy().astype(np.float64)
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    ref = orc.diff_grad(d, spp, dimage)
    assert g.shape == ref.shape == (dr.n_params,)
    err = np.abs(g - ref)
    tol = GRAD_ABS * np.abs(ref).max() + GRAD_REL * np.abs(ref)
    worst = int(np.argmax(err / tol))
    assert np.all(err <= tol), f"param {worst}: gpu {g[worst]:.6g} oracle {ref[worst]:.6g}"
    assert np.abs(ref).max() > 0


def test_backward_matches_central_differences(zgl_lib, cuda):
    """h = 1e-3, common random numbers; baseColor, specular and light power."""
    import torch

    d = diff_scene(seed=24, width=32, height=32)
    spp, params = 4, dict(max_depth=6)
    sc, dr, dimage, dimg_t = _setup(d, spp, params)
    p0 = dr.params()
    dr.forward()
    g = dr.backward(dimg_t).cpu().numpy().astype(np.float64)
    img = torch.empty((32, 32, 3), dtype=torch.float32, device="cuda")

    def loss(p):
        dr.set_params(p)
        dr.forward(out=img)
        return float((img.double() * dimg_t.double()).sum())

    slots = [0, 1, 2, 5, 14, 30, 31, 32, 41, 48, 49, 50]
    for slot in slots:
        h = 1e-3 * max(1.0, abs(float(p0[slot])))
        pp, pm = p0.copy(), p0.copy()
        pp[slot] += np.float32(h)
        pm[slot] -= np.float32(h)
        hh = (float(pp[slot]) - float(pm[slot])) / 2
        fd = (loss(pp) - loss(pm)) / (2 * hh)
        assert abs(g[slot] - fd) <= 5e-3 * max(abs(fd), 1e-2 * np.abs(g).max()), \
            f"slot {slot}: adjoint {g[slot]:.6g} fd {fd:.6g}"
    dr.set_params(p0)
    assert np.array_equal(dr.params(), p0)


class _Render:
    """torch.autograd.Function over DiffRenderer (test harness only)."""

    @staticmethod
    def make(dr):
        import torch

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, p):
                dr.set_params(p.detach().contiguous())
                return dr.forward()

            @staticmethod
            def backward(ctx, grad_img):
                return dr.backward(grad_img.contiguous())

        return Fn.apply


def test_autograd_inverse_rendering_reduces_the_loss(zgl_lib, cuda):
    import torch

    from zillumgl_gb300.synthetic import perturbed_params

    d = diff_scene(seed=25, width=48, height=48)
    sc = Scene(d)
    dr = DiffRenderer(sc, 4, max_depth=4)
    p_true = dr.params()
    target = dr.forward().clone()
    p = torch.tensor(perturbed_params(p_true, 8, seed=26), device="cuda", requires_grad=True)
    render = _Render.make(dr)
    opt = torch.optim.Adam([p], lr=0.02)
    losses = []
    for _ in range(25):
        opt.zero_grad()
        img = render(p)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            p.clamp_(0.01, 100.0)
        losses.append(float(loss.detach()))
    assert losses[-1] < 0.5 * losses[0], losses
    err0 = np.abs(perturbed_params(p_true, 8, seed=26) - p_true)[:48].mean()
    err1 = np.abs(p.detach().cpu().numpy() - p_true)[:48].mean()
    assert err1 < err0


def test_parameter_validation(zgl_lib, cuda):
    d = diff_scene(seed=27, width=16, height=16)
    sc = Scene(d)
    dr = DiffRenderer(sc, 1)
    p = dr.params()
    assert p.shape == (51,)
    assert np.allclose(p[48:], 15.0)
    bad = p.copy()
    bad[49] = -1.0
    with pytest.raises(ZglError):
        dr.set_params(bad)
    assert np.array_equal(dr.params(), p)
    bad = p.copy()
    bad[3] = np.nan
    with pytest.raises(ZglError):
        dr.set_params(bad)
    with pytest.raises(ValueError):
        dr.set_params(p[:10])
    with pytest.raises(ZglError):
        DiffRenderer(sc, 0)
    # the scene itself sees new values: the light's power doubles the image
    img1 = dr.forward().clone()
    q = p.copy()
    q[48:] *= 2
    dr.set_params(q)
    img2 = dr.forward()
    assert np.allclose(img2.cpu().numpy(), 2 * img1.cpu().numpy(), rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("spp,depth", [(32, 6), (3, 4), (40, 5), (4, 11)])
def test_fused_l2_step_equals_forward_then_backward(zgl_lib, cuda, spp, depth):
    """zgl_diff_step_l2: the image equals zgl_diff_forward's bit for bit, the
    loss the mean squared error, and the gradient zgl_diff_backward's for
    dL/dimage = 2 (image - target) / numel up to the order of the float
    atomics (relative 5e-5 of the largest component); several sample
    counts, and paths deeper than the 9 kept ray casts (traced again)."""
    import torch

    d = diff_scene(seed=28, width=24, height=20)
    params = dict(max_depth=depth, russian_roulette=1, rr_start_depth=3) if depth > 8 else dict(max_depth=depth)
    sc = Scene(d)
    dr = DiffRenderer(sc, spp, **params)
    rng = np.random.default_rng(29)
    target = torch.from_numpy(rng.uniform(0.0, 0.6, (20, 24, 3)).astype(np.float32)).cuda()
    img, grad, loss = dr.step_l2(target)
    torch.cuda.synchronize()
    ref_img = dr.forward()
    assert torch.equal(img.view(torch.int32), ref_img.view(torch.int32))
    diff = ref_img - target
    ref_loss = float((diff.double() ** 2).mean())
    assert abs(float(loss) - ref_loss) <= 1e-5 * ref_loss
    ref_grad = dr.backward(diff * (2.0 / diff.numel())).cpu().numpy().astype(np.float64)
    g = grad.cpu().numpy().astype(np.float64)
    assert np.abs(g - ref_grad).max() <= 5e-5 * np.abs(ref_grad).max() + 1e-12, \
        f"max diff {np.abs(g - ref_grad).max():.3g} of {np.abs(ref_grad).max():.3g}"
    assert np.abs(ref_grad).max() > 0
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    dimg = (diff * (2.0 / diff.numel())).cpu().numpy()
    o = orc.diff_grad(d, spp, dimg)
    tol = GRAD_ABS * np.abs(o).max() + GRAD_REL * np.abs(o)
    assert np.all(np.abs(g - o) <= tol)
    dr.close()
    sc.close()


@pytest.mark.parametrize("depth", [6, 11])
def test_replay_from_kept_casts_equals_traced_replay(zgl_lib, cuda, depth):
    """zgl_diff_backward replays the paths from the ray casts zgl_diff_forward
    kept; after zgl_diff_set_params (same values) the casts are dropped and
    every ray is traced again.  Both gradients agree up to the order of the
    float atomics (relative 5e-5 of the largest component), with the
    full-material scene and paths deeper than the 9 kept casts."""
    import torch

    d = diff_scene(seed=31, width=40, height=24)
    params = dict(max_depth=depth, russian_roulette=1, rr_start_depth=3) if depth > 8 else dict(max_depth=depth)
    sc = Scene(d)
    dr = DiffRenderer(sc, 8, **params)
    img = dr.forward()
    rng = np.random.default_rng(32)
    dimg = torch.from_numpy(rng.uniform(-1e-3, 1e-3, tuple(img.shape)).astype(np.float32)).cuda()
    g_kept = dr.backward(dimg).cpu().numpy().astype(np.float64)
    dr.set_params(dr.params())
    g_traced = dr.backward(dimg).cpu().numpy().astype(np.float64)
    assert np.abs(g_kept).max() > 0
    assert np.abs(g_kept - g_traced).max() <= 5e-5 * np.abs(g_traced).max() + 1e-12
    dr.close()
    sc.close()


def test_roughness_and_metallic_match_frozen_sampling_differences(zgl_lib, cuda):
    """The GPU adjoint's roughness (raw, before the remap of
    material_loader.glsl:46) and metallic (which also steers the lobe pick,
    material.glsl:537-540) derivatives against central differences
    (h = 1e-3) of the oracle's frozen-sampling estimator: every sampling
    decision taken at the unperturbed parameters, only the BSDF values
    moved, which is the estimator a detached-sampling adjoint
    differentiates."""
    d = diff_scene(seed=24, width=32, height=32)
    spp, params = 4, dict(max_depth=6)
    sc, dr, dimage, dimg_t = _setup(d, spp, params)
    dr.forward()
    g = dr.backward(dimg_t).cpu().numpy().astype(np.float64)
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    W, H = d.film

    def loss(materials):
        img = orc.render_pt_frozen(materials, np.arange(W * H), spp).astype(np.float64) / spp
        return float(np.sum(img.reshape(H, W, 3) * dimage))

    nmat = d.materials.shape[0]
    for m in range(nmat):
        for slot, col in ((6 * m + 3, 3), (6 * m + 4, 5)):
            h = 1e-3 * max(1.0, abs(float(d.materials[m, col])))
            mp, mm = d.materials.copy(), d.materials.copy()
            mp[m, col] += np.float32(h)
            mm[m, col] -= np.float32(h)
            hh = (float(mp[m, col]) - float(mm[m, col])) / 2
            fd = (loss(mp) - loss(mm)) / (2 * hh)
            assert abs(g[slot] - fd) <= 5e-3 * max(abs(fd), 1e-2 * np.abs(g).max()), \
                f"slot {slot}: adjoint {g[slot]:.6g} frozen fd {fd:.6g}"
    dr.close()
    sc.close()
