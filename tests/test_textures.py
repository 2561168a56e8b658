"""Albedo textures on the CPU: the oracle's texture lookup against an
independent numpy restatement of the GL rules it follows
(material_loader.glsl:14-15 and Texture.cpp:134-171: level 0, GL_LINEAR
magnification, GL_REPEAT over the whole layer, sRGB decoded per texel), the
scene's texture tables, and the scene's input checks."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import ZglError
from zillumgl_gb300.scene import Scene, mat_tex
from zillumgl_gb300.synthetic import textured_scene, texture_images


def _srgb_to_linear():
    c = np.arange(256) / 255.0
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)


def _numpy_sample(layers, scale, tex, uv):
    """GL 4.5 section 8.14.2 linear filtering, evaluated in float32."""
    f = np.float32
    lut = _srgb_to_linear()
    H, W = layers.shape[1], layers.shape[2]
    u0 = uv[:, 0].astype(f)
    v0 = uv[:, 1].astype(f)
    s = (u0 - np.floor(u0)).astype(f) * scale[tex, 0]
    t = (v0 - np.floor(v0)).astype(f) * scale[tex, 1]
    u = (s * f(W)).astype(f) - f(0.5)
    v = (t * f(H)).astype(f) - f(0.5)
    a = (u - np.floor(u)).astype(f)
    b = (v - np.floor(v)).astype(f)
    i0 = np.floor(u).astype(np.int64) % W
    j0 = np.floor(v).astype(np.int64) % H
    i1, j1 = (i0 + 1) % W, (j0 + 1) % H
    T = lambda i, j: lut[layers[tex, j, i]]  # noqa: E731
    one = f(1.0)
    w00, w10 = ((one - a) * (one - b))[:, None], (a * (one - b))[:, None]
    w01, w11 = ((one - a) * b)[:, None], (a * b)[:, None]
    return ((w00 * T(i0, j0) + w10 * T(i1, j0)) + w01 * T(i0, j1)) + w11 * T(i1, j1)


def test_oracle_texture_lookup_matches_gl_rules():
    d = textured_scene(width=8, height=8)
    orc = oracle.OracleScene(d, np.zeros((256, 32), np.uint32), {})
    layers, scale = oracle.texture_layers(d.textures)
    rng = np.random.default_rng(3)
    uv = np.concatenate([rng.uniform(-3, 3, (4000, 2)),
                         np.array([[0, 0], [1, 1], [-1e-9, 0.5], [0.999999, 0.25], [2.0, -2.0], [0.5, 1e-8]])])
    uv = uv.astype(np.float32)
    for tex in range(3):
        got = orc.texture_sample(tex, uv)
        ref = _numpy_sample(layers, scale, tex, uv)
        assert np.array_equal(got.view(np.uint32), ref.astype(np.float32).view(np.uint32)), tex
    # texel centres of the largest image return the decoded texel exactly
    img = d.textures[2]
    H, W = img.shape[:2]
    ys, xs = np.mgrid[0:H, 0:W]
    uv = np.stack([(xs.ravel() + 0.5) / W, (ys.ravel() + 0.5) / H], 1).astype(np.float32)
    got = orc.texture_sample(2, uv)
    assert np.allclose(got, _srgb_to_linear()[img.reshape(-1, 3)], rtol=0, atol=1e-6)


def test_scene_texture_tables(zgl_lib):
    d = textured_scene(width=8, height=8)
    sc = Scene(d, host_only=True)
    layers, scale = oracle.texture_layers(d.textures)
    assert np.array_equal(sc.export("tex_scale").reshape(3, 2), scale)
    assert np.array_equal(sc.export("srgb_lut").view(np.uint32),
                          _srgb_to_linear().view(np.uint32))
    assert layers.shape == (3, 64, 64, 3)
    sc.close()


@pytest.mark.parametrize("bad", ["index", "below", "size", "texcoord"])
def test_scene_rejects_invalid_textures(zgl_lib, bad):
    d = textured_scene(width=8, height=8)
    if bad == "index":
        d.obj_mat_tex[0] = mat_tex(0, 3)
    elif bad == "below":
        d.obj_mat_tex[0] = mat_tex(0, -2)
    elif bad == "size":
        d.textures[1] = np.zeros((0, 4, 3), np.uint8)
    else:
        d.obj_texcoords[3, 1] = np.inf
    with pytest.raises(ZglError) as e:
        Scene(d, host_only=True)
    assert e.value.status == 1


def test_texture_images_are_seeded():
    a, b = texture_images(5), texture_images(5)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert [t.shape for t in a] == [(24, 40, 3), (17, 31, 3), (64, 64, 3)]
