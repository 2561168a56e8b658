"""Host sampling tables (CPU): product vs oracle vs the reference's own code.

* Light alias tables: AliasTable::build (src/math/AliasTable.h:12-54) — the
  product and the oracle reproduce the golden vectors recorded from the
  reference header (tests/golden/make_golden.py), and the header itself when
  the reference tree is present.
* Sobol generator matrices: regenerated from direction numbers, equal to the
  reference's 256x32 table (SHA-256 and sample dimensions).
* Light power split, environment alias tables, RGB16F texels, noise texture,
  per-pixel seeds and camera uniforms: product and oracle bit for bit.
"""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from zillumgl_gb300.scene import LAMBERTIAN, PRINCIPLED, Scene, alias_table, mat_tex, material
from zillumgl_gb300.synthetic import cornell_scene, sky_environment

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_tables.json").read_text())


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", sorted(GOLDEN["alias"]))
def test_alias_table_matches_reference_golden(zgl_lib, name):
    case = GOLDEN["alias"][name]
    pdf = np.array(case["pdf"], np.uint32).view(np.float32)
    alias, prob = alias_table(pdf)
    assert alias.tolist() == case["alias"]
    assert _bits(prob).tolist() == case["prob_bits"]
    oa, op = oracle.alias_build(pdf)
    assert oa.tolist() == case["alias"] and _bits(op).tolist() == case["prob_bits"]


def test_alias_table_matches_reference_header_random(zgl_lib):
    rng = np.random.default_rng(5)
    for n in (1, 2, 3, 17, 1000):
        pdf = rng.lognormal(0, 1.5, n).astype(np.float32)
        pdf[rng.random(n) < 0.2] = 0.0
        if pdf.sum() == 0:
            pdf[0] = 1.0
        ref = oracle.ref_alias_build(pdf)
        if ref is None:
            pytest.skip("reference tree not present (golden vectors cover this case)")
        a, p = alias_table(pdf)
        assert np.array_equal(a, ref[0]) and np.array_equal(_bits(p), _bits(ref[1]))


def test_alias_table_distribution():
    pdf = np.array([1.0, 3.0, 0.0, 6.0], np.float32)
    alias, prob = alias_table(pdf)
    mass = np.zeros(4)
    for i in range(4):
        mass[i] += prob[i] / 4
        mass[alias[i]] += (1 - prob[i]) / 4
    assert np.allclose(mass, pdf / pdf.sum(), atol=1e-6)


def test_sobol_matrices_equal_reference_table(zgl_lib):
    sc = Scene(cornell_scene(width=8, height=8), host_only=True)
    mats = sc.export("sobol")
    assert hashlib.sha256(mats.tobytes()).hexdigest() == GOLDEN["sobol"]["sha256"]
    for d, cols in GOLDEN["sobol"]["dims"].items():
        assert mats[int(d) * 32:(int(d) + 1) * 32].tolist() == cols
    # dimension 0 is the van der Corput (bit reversal) sequence
    assert mats[:32].tolist() == [1 << (31 - i) for i in range(32)]


def _multi_light_scene(env=True, w=24, h=16):
    d = cornell_scene(seed=3, width=w, height=h)
    # two light instances: the ceiling quad and a small triangle fan
    lv = np.concatenate([d.light_vertices, np.array([[0.9, 0.9, 0.5], [0.95, 0.9, 0.5], [0.9, 0.95, 0.6]],
                                                     np.float32)])
    ln = np.concatenate([d.light_normals, np.tile(np.array([[-1.0, 0.0, 0.0]], np.float32), (3, 1))])
    li = np.concatenate([d.light_indices, np.array([4, 5, 6], np.uint32)])
    d.light_vertices, d.light_normals, d.light_indices = lv, ln, li
    d.light_first = np.array([0, 2, 3], np.uint32)
    d.light_power = np.array([[15.0, 15.0, 15.0], [2.0, 1.0, 0.5]], np.float32)
    if env:
        d.env_rgb = sky_environment(64, 32, seed=4)
        d.env_rotation = 0.3
    return d.normalized()


def test_scene_tables_match_oracle(zgl_lib):
    d = _multi_light_scene()
    sc = Scene(d, host_only=True)
    lp, la, lpr, lsum = oracle.light_tables(d)
    assert np.array_equal(_bits(sc.export("light_power")), _bits(lp.reshape(-1)))
    assert np.array_equal(sc.export("light_alias"), la)
    assert np.array_equal(_bits(sc.export("light_prob")), _bits(lpr))
    sca = sc.export("scalars")
    assert _bits(sca[:1])[0] == _bits(np.array([lsum], np.float32))[0]
    ea, ep, esum = oracle.env_tables(d.env_rgb)
    assert np.array_equal(sc.export("env_alias"), ea)
    assert np.array_equal(_bits(sc.export("env_prob")), _bits(ep))
    assert sca[1] == np.float32(int(esum)), "envSum is the int-truncated pdf sum (EnvironmentMap.h:22)"
    half = d.env_rgb.astype(np.float16).astype(np.float32).reshape(-1)
    assert np.array_equal(_bits(sc.export("env_texels")), _bits(half))
    assert np.array_equal(_bits(sc.export("noise")), _bits(oracle.noise(*d.film)))
    assert np.array_equal(_bits(sc.export("camera")), _bits(oracle.camera(d.cam_angle, d.cam_fov)))


def test_noise_engine_is_minstd_rand0():
    # libstdc++ default_random_engine: x1 = 16807, x2 = 16807^2 mod (2^31 - 1)
    n = oracle.noise(2, 1)
    x1, x2 = 16807, (16807 * 16807) % 2147483647
    assert n[0] == np.float32(np.float32(x1 - 1) / np.float32(2147483646.0))
    assert n[1] == np.float32(np.float32(x2 - 1) / np.float32(2147483646.0))


def test_camera_basis_is_orthonormal_and_z_up():
    cam = oracle.camera((30.0, 10.0, 0.0), 60.0)
    f, r, u = cam[0:3], cam[3:6], cam[6:9]
    for a in (f, r, u):
        assert abs(np.linalg.norm(a) - 1) < 1e-6
    assert abs(f @ r) < 1e-6 and abs(f @ u) < 1e-6 and abs(r @ u) < 1e-6
    assert u[2] > 0 and abs(cam[18] - np.tan(np.radians(30))) < 1e-6
    inv = cam[9:18].reshape(3, 3).T  # column-major
    m = np.stack([r, u, f], axis=1)
    assert np.allclose(inv @ m, np.eye(3), atol=1e-5)


def test_env_sum_truncation_and_leftover_probabilities():
    rgb = np.full((4, 8, 3), 0.1, np.float32)
    rgb[1, 3] = 50.0
    alias, prob, s = oracle.env_tables(rgb)
    W = 8
    rows = prob.reshape(4, W + 1)
    assert np.all(rows[:, :W] <= 1.0)
    assert np.all((rows[:, :W] == 1.0) == (alias.reshape(4, W + 1)[:, :W] == np.arange(W)))
    assert s > 0 and np.float32(int(s)) <= s


@pytest.mark.parametrize("bad", ["texture", "type", "ior", "nan", "index", "power", "film"])
def test_scene_rejects_invalid_input(zgl_lib, bad):
    from zillumgl_gb300 import ZglError

    d = cornell_scene(width=8, height=8)
    if bad == "texture":
        d.obj_mat_tex[0] = mat_tex(0, 2)
    elif bad == "type":
        d.materials[0] = material(7)
    elif bad == "ior":
        d.materials[0] = material(3, ior=0.0)
    elif bad == "nan":
        d.materials[0, 0] = np.nan
    elif bad == "index":
        d.obj_indices[5] = 10 ** 6
    elif bad == "power":
        d.light_power[:] = 0.0
    elif bad == "film":
        d.film = (0, 8)
    with pytest.raises(ZglError) as e:
        Scene(d, host_only=True)
    assert e.value.status == 1


def test_transcendentals_accuracy():
    rng = np.random.default_rng(0)
    x = rng.uniform(-20, 20, 200000).astype(np.float32)
    x64 = x.astype(np.float64)

    def ulps(got, ref):
        sp = np.spacing(np.abs(ref.astype(np.float32))).astype(np.float64)
        return np.abs(got.astype(np.float64) - ref) / np.maximum(sp, np.finfo(np.float32).tiny)

    assert ulps(oracle.transc(0, x), np.sin(x64)).max() <= 4
    assert ulps(oracle.transc(1, x), np.cos(x64)).max() <= 4
    y = rng.standard_normal(200000).astype(np.float32)
    assert ulps(oracle.transc(2, y, x), np.arctan2(y.astype(np.float64), x64)).max() <= 4
    z = np.exp(rng.uniform(-80, 80, 200000)).astype(np.float32)
    assert ulps(oracle.transc(3, z), np.log(z.astype(np.float64))).max() <= 4
    w = rng.uniform(-140, 127, 200000).astype(np.float32)
    assert ulps(oracle.transc(4, w), np.exp2(w.astype(np.float64))).max() <= 4
    a = rng.uniform(1e-4, 1, 100000).astype(np.float32)
    b = rng.uniform(0, 1, 100000).astype(np.float32)
    ref = np.power(a.astype(np.float64), b)
    assert (np.abs(oracle.transc(5, a, b) - ref) / ref).max() < 4e-6
    # special values
    assert oracle.transc(2, np.array([0.0, -0.0], np.float32), np.array([-1.0, -1.0], np.float32)).tolist() == \
        [np.float32(np.pi), -np.float32(np.pi)]
    assert np.isnan(oracle.transc(3, np.array([-1.0], np.float32))[0])
    assert oracle.transc(3, np.array([0.0], np.float32))[0] == -np.inf
