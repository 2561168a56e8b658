"""Scene XML loading (Scene::load, src/core/Scene.cpp:58-127): host-side
parsing, model transforms (Model.cpp:62-71), material records
(MaterialLoader.cpp:5-68), light instances and the environment map."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import ZglError
from zillumgl_gb300.scene import Scene

CUBE = """# unit cube without normals, faces wound counter-clockwise from outside
# (smooth normals are generated from the winding)
v -0.5 -0.5 -0.5
v 0.5 -0.5 -0.5
v 0.5 0.5 -0.5
v -0.5 0.5 -0.5
v -0.5 -0.5 0.5
v 0.5 -0.5 0.5
v 0.5 0.5 0.5
v -0.5 0.5 0.5
f 1 4 3 2
f 5 6 7 8
f 1 2 6 5
f 2 3 7 6
f 3 4 8 7
f 4 1 5 8
"""
QUAD = """v -1 -1 0
v 1 -1 0
v 1 1 0
v -1 1 0
vn 0 0 1
f 1//1 2//1 3//1 4//1
"""
SCENE = """<?xml version="1.0"?>
<scene name="t">
  <integrator type="path"><maxBounce value="3"/><size width="40" height="24"/></integrator>
  <sampler type="sobol"><numSamples value="16"/></sampler>
  <camera type="thinLens">
    <position value="0 -6 2"/><angle value="0 -5 0"/><fov value="50"/>
    <lensRadius value="0"/><focalDistance value="1"/>
  </camera>
  <modelInstances>
    <!-- floor -->
    <modelInstance path="quad.obj" name="floor" type="object">
      <transform translate="0 0 0" scale="4 4 1" rotate="0 -90 0"/>
      <material type="lambertian"><baseColor value="0.6 0.5 0.4"/></material>
    </modelInstance>
    <modelInstance path="cube.obj" name="box" type="object">
      <transform translate="0.3 0.2 0.5" scale="1 1 1" rotate="30 0 0"/>
      <material type="principled">
        <baseColor value="0.2 0.7 0.3"/><roughness value="0.4"/><metallic value="1"/><clearcoat value="0.5"/>
      </material>
    </modelInstance>
    <modelInstance path="quad.obj" name="lamp" type="light">
      <transform translate="0 0 3" scale="0.5 0.5 1" rotate="0 90 0"/>
      <radiance value="20 18 16"/>
    </modelInstance>
  </modelInstances>
  <envMap path="sky.pfm"/>
</scene>
"""


def _write(tmp_path, scene=SCENE, env=True):
    (tmp_path / "cube.obj").write_text(CUBE)
    (tmp_path / "quad.obj").write_text(QUAD)
    (tmp_path / "scene.xml").write_text(scene)
    if env:
        H, W = 8, 16
        img = np.linspace(0.1, 2.0, H * W * 3, dtype=np.float32).reshape(H, W, 3)
        with open(tmp_path / "sky.pfm", "wb") as f:
            f.write(f"PF\n{W} {H}\n-1.0\n".encode())
            f.write(img[::-1].astype("<f4").tobytes())  # PFM stores the bottom row first
        return img
    return None


def _rot(axis, deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    x, y, z = axis
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                     [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                     [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])


def _model(t, sc, r):
    # translate * scale * rotX(90) * rotZ(r0) * rotX(r1) * rotY(r2)
    m = np.diag(sc) @ _rot((1, 0, 0), 90) @ _rot((0, 0, 1), r[0]) @ _rot((1, 0, 0), r[1]) @ _rot((0, 1, 0), r[2])
    return m, np.asarray(t, float)


def test_xml_scene_tables(zgl_lib, tmp_path):
    img = _write(tmp_path)
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    info = sc.info
    assert sc.film == (40, 24)
    assert info["obj_triangles"] == 2 + 12 and info["light_triangles"] == 2 and info["materials"] == 2
    assert (info["env_w"], info["env_h"]) == (16, 8)
    v = sc.export("vertices").reshape(-1, 3)
    # floor quad: corners at (+-4, +-4) in the z = 0 plane after the transform
    m, t = _model((0, 0, 0), (4, 4, 1), (0, -90, 0))
    quad = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], float)
    assert np.allclose(v[:4], quad @ m.T + t, atol=1e-5)
    assert np.allclose(np.abs(v[:4, 2]), 0, atol=1e-5)
    # box: 8 joined corners, rotated 30 degrees about z after the fixed +90 about x
    m, t = _model((0.3, 0.2, 0.5), (1, 1, 1), (30, 0, 0))
    cube = np.array([[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [0.5, 0.5, -0.5], [-0.5, 0.5, -0.5],
                     [-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [0.5, 0.5, 0.5], [-0.5, 0.5, 0.5]])
    assert np.allclose(np.sort(v[4:12], axis=0), np.sort(cube @ m.T + t, axis=0), atol=1e-5)
    n = sc.export("normals").reshape(-1, 3)
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-5)
    # floor normal is +z after the transform; cube normals point outwards
    assert np.allclose(n[:4], [0, 0, 1], atol=1e-5)
    centre = v[4:12].mean(0)
    assert np.all(np.sum((v[4:12] - centre) * n[4:12], axis=1) > 0)
    mats = sc.export("materials").reshape(-1, 16)
    assert np.allclose(mats[0, :3], [0.6, 0.5, 0.4]) and mats[0, 13:14].view(np.int32)[0] == 0
    assert np.allclose(mats[1, :4], [0.2, 0.7, 0.3, 0.4]) and mats[1, 5] == 1.0 and mats[1, 10] == 0.5
    assert mats[1, 13:14].view(np.int32)[0] == 1
    assert mats[1, 6] == 1.0 and mats[1, 12] == np.float32(1.5)  # Material.h defaults kept
    mt = sc.export("mat_tex")
    assert np.all((mt & 0xFFFF)[:2] == 0) and np.all((mt & 0xFFFF)[2:] == 1) and np.all((mt >> 16) == -1)
    # light power split by area over the lamp's two triangles (Scene.cpp:200-243)
    lp = sc.export("light_power").reshape(-1, 3)
    assert np.allclose(lp.sum(0), [20, 18, 16], rtol=1e-6)
    # camera uniforms as Camera::update computes them
    assert np.array_equal(sc.export("camera"), oracle.camera((0, -5, 0), 50))
    # environment: rows top first, RGB16F-rounded
    assert np.array_equal(sc.export("env_texels"), img.astype(np.float16).astype(np.float32).reshape(-1))
    sc.close()


@pytest.mark.parametrize("broken", ["unclosed", "no_scene", "missing_model", "bad_face"])
def test_xml_errors_are_parse_status(zgl_lib, tmp_path, broken):
    text = SCENE
    if broken == "unclosed":
        text = SCENE.replace("</modelInstances>", "")
    elif broken == "no_scene":
        text = "<?xml version='1.0'?><world/>"
    elif broken == "missing_model":
        text = SCENE.replace("cube.obj", "nothing.obj")
    _write(tmp_path, text)
    if broken == "bad_face":
        (tmp_path / "cube.obj").write_text("v 0 0 0\nv 1 0 0\nf 1 2 9\n")
    with pytest.raises(ZglError) as e:
        Scene.load(tmp_path / "scene.xml", host_only=True)
    assert e.value.status == 5


def test_xml_without_env_is_black(zgl_lib, tmp_path):
    _write(tmp_path, SCENE.replace('<envMap path="sky.pfm"/>', ""), env=False)
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    assert sc.info["env_w"] == 0 and sc.export("scalars")[1] == 0.0
    sc.close()


# ---------------------------------------------------------------- textures
TEX_OBJ = """mtllib tex.mtl
v -1 -1 0
v 1 -1 0
v 1 1 0
v -1 1 0
v 3 -1 0
v 3 1 0
vt 0 0
vt 2 0
vt 2 2
vt 0 2
vt 0.25 0.75
vn 0 0 1
usemtl checker
f 1/1/1 2/2/1 3/3/1 4/4/1
usemtl noise
f 2/1/1 5/2/1 6/3/1
f 2/5/1 6/3/1 3/4/1
usemtl plain
f 4/1/1 3/2/1 6/5/1
"""
TEX_MTL = """newmtl checker
Kd 0.9 0.1 0.2
map_Kd -s 1 1 1 checker.ppm
newmtl noise
Kd 0.3 0.4 0.5
map_Kd noise.bmp
newmtl plain
Kd 0.25 0.5 0.75
"""
TEX_SCENE = """<?xml version="1.0"?>
<scene>
  <integrator type="path"><size width="32" height="24"/></integrator>
  <sampler type="sobol"/>
  <camera type="thinLens"><position value="1 -3.5 3"/><angle value="0 -45 0"/><fov value="60"/>
    <lensRadius value="0"/><focalDistance value="1"/></camera>
  <modelInstances>
    <modelInstance path="tex.obj" type="object">
      <transform translate="0 0 0" scale="1 1 1" rotate="0 -90 0"/>
      <material type="default"/>
    </modelInstance>
    <modelInstance path="tex.obj" type="object">
      <transform translate="0 0 0.5" scale="1 1 1" rotate="0 -90 0"/>
      MATERIAL
    </modelInstance>
    <modelInstance path="quad.obj" type="light">
      <transform translate="0 0 3" scale="1 1 1" rotate="0 90 0"/>
      <radiance value="30 30 30"/>
    </modelInstance>
  </modelInstances>
</scene>
"""


def _bmp24(img):
    """Uncompressed 24-bit BMP, bottom row first, rows padded to 4 bytes."""
    import struct

    H, W = img.shape[:2]
    stride = (W * 3 + 3) & ~3
    rows = b"".join(img[y, :, ::-1].tobytes() + b"\0" * (stride - 3 * W) for y in range(H - 1, -1, -1))
    head = struct.pack("<2sIHHI", b"BM", 54 + len(rows), 0, 0, 54)
    info = struct.pack("<IiiHHIIiiII", 40, W, H, 1, 24, 0, len(rows), 2835, 2835, 0, 0)
    return head + info + rows


def _write_textured(tmp_path, material='<material type="principled"><roughness value="0.5"/></material>'):
    rng = np.random.default_rng(9)
    checker = np.where(((np.add.outer(np.arange(6), np.arange(10)) % 2)[..., None]) == 0,
                       np.array([230, 20, 40], np.uint8), np.array([10, 200, 90], np.uint8)).astype(np.uint8)
    noise = rng.integers(0, 256, (5, 7, 3)).astype(np.uint8)
    (tmp_path / "checker.ppm").write_bytes(b"P6\n# a comment\n10 6\n255\n" + checker.tobytes())
    (tmp_path / "noise.bmp").write_bytes(_bmp24(noise))
    (tmp_path / "tex.obj").write_text(TEX_OBJ)
    (tmp_path / "tex.mtl").write_text(TEX_MTL)
    (tmp_path / "quad.obj").write_text(QUAD)
    (tmp_path / "scene.xml").write_text(TEX_SCENE.replace("MATERIAL", material))
    return [checker, noise]


def test_obj_textures_materials_and_texcoords(zgl_lib, tmp_path):
    _write_textured(tmp_path)
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    i = sc.info
    assert i["textures"] == 2 and i["obj_triangles"] == 2 * 5 and i["materials"] == 2 * 3
    mats = sc.export("materials").reshape(-1, 16)
    # "default": each usemtl slot takes its Kd on Material's defaults (Lambertian)
    assert np.allclose(mats[:3, :3], [[0.9, 0.1, 0.2], [0.3, 0.4, 0.5], [0.25, 0.5, 0.75]])
    assert np.all(mats[:3, 13:14].view(np.int32) == 0)
    # an explicit material replaces every slot's parameters (Scene.cpp:47-53)
    assert np.all(mats[3:, 13:14].view(np.int32) == 1) and np.allclose(mats[3:, 3], 0.5)
    mt = sc.export("mat_tex")
    # textures follow the slots and are shared between the two instances
    assert (mt & 0xFFFF).tolist() == [0, 0, 1, 1, 2, 3, 3, 4, 4, 5]
    assert (mt >> 16).tolist() == [0, 0, 1, 1, -1, 0, 0, 1, 1, -1]
    # texcoords: v flipped (aiProcess_FlipUVs), corners joined on (v, vt, vn)
    uv = sc.export("texcoords").reshape(-1, 2)
    assert i["obj_vertices"] == 2 * 12  # 12 distinct (v, vt, vn) corners per instance
    assert {tuple(x) for x in uv[:12].tolist()} == {(0.0, 1.0), (2.0, 1.0), (2.0, -1.0), (0.0, -1.0), (0.25, 0.25)}
    scale = sc.export("tex_scale").reshape(-1, 2)
    assert np.array_equal(scale, np.array([[1.0, 1.0], [np.float32(7) / np.float32(10), np.float32(5) / np.float32(6)]],
                                          np.float32))
    sc.close()


def test_missing_or_unreadable_texture_leaves_faces_untextured(zgl_lib, tmp_path):
    _write_textured(tmp_path)
    (tmp_path / "noise.bmp").write_bytes(b"BM not an image")
    (tmp_path / "checker.ppm").unlink()
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    assert sc.info["textures"] == 0 and np.all((sc.export("mat_tex") >> 16) == -1)
    sc.close()


def _bmp32_top_down(img):
    """Uncompressed 32-bit BMP with a negative height (rows top first)."""
    import struct

    H, W = img.shape[:2]
    bgra = np.concatenate([img[..., ::-1], np.full((H, W, 1), 255, np.uint8)], -1)
    rows = bgra.tobytes()
    head = struct.pack("<2sIHHI", b"BM", 54 + len(rows), 0, 0, 54)
    info = struct.pack("<IiiHHIIiiII", 40, W, -H, 1, 32, 0, len(rows), 2835, 2835, 0, 0)
    return head + info + rows


def test_image_variants_and_default_material(zgl_lib, tmp_path):
    """ASCII PPM (maxval 100, rescaled), top-down 32-bit BMP, and an OBJ
    without a material library (assimp's default material: diffuse 0.6)."""
    _write_textured(tmp_path)
    rng = np.random.default_rng(3)
    small = rng.integers(0, 101, (3, 4, 3))
    txt = "P3\n4 3\n100\n" + " ".join(str(int(x)) for x in small.reshape(-1)) + "\n"
    (tmp_path / "checker.ppm").write_text(txt)
    big = rng.integers(0, 256, (9, 12, 3)).astype(np.uint8)
    (tmp_path / "noise.bmp").write_bytes(_bmp32_top_down(big))
    (tmp_path / "plain.obj").write_text(QUAD)
    scene = TEX_SCENE.replace("MATERIAL", '<material type="default"/>').replace(
        '<modelInstance path="quad.obj" type="light">',
        '<modelInstance path="plain.obj" type="object"><transform translate="0 0 -1"/>'
        '<material type="default"/></modelInstance>\n    <modelInstance path="quad.obj" type="light">')
    (tmp_path / "scene.xml").write_text(scene)
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    assert sc.info["textures"] == 2
    # sizes 4x3 and 12x9: scales relative to the 12x9 layer
    scale = sc.export("tex_scale").reshape(-1, 2)
    assert np.array_equal(scale, np.array([[np.float32(4) / np.float32(12), np.float32(3) / np.float32(9)],
                                           [1.0, 1.0]], np.float32))
    tex = sc.export("tex_texels").reshape(2, 9, 12)
    rgb = np.stack([tex & 255, (tex >> 8) & 255, (tex >> 16) & 255], -1).astype(np.int64)
    assert np.array_equal(rgb[0, :3, :4], (small * 255 + 50) // 100)  # maxval 100 rescaled to 255
    assert np.all(rgb[0, 3:] == 0) and np.all(rgb[0, :, 4:] == 0)  # rest of the layer zero
    assert np.array_equal(rgb[1], big)  # top-down BMP rows kept in order
    mats = sc.export("materials").reshape(-1, 16)
    assert np.allclose(mats[-1, :3], 0.6)  # the OBJ without .mtl
    assert (sc.export("mat_tex")[-2:] >> 16).tolist() == [-1, -1]
    sc.close()


def test_obj_edge_cases(zgl_lib, tmp_path):
    """Unknown usemtl names and a missing .mtl fall back to the default
    material (diffuse 0.6); `vt u` alone means v = 0 (flipped to 1);
    negative face indices count back from the last vertex / texcoord;
    a bad corner token is a parse error."""
    obj = """mtllib missing.mtl
v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0
vt 0.25
vt 0.5 0.5
vn 0 0 1
usemtl nowhere
f -4/-2/-1 -3/-1/-1 -2/-1/-1
usemtl nowhere
f 2/1/1 4/2/1 3/2/1
"""
    (tmp_path / "edge.obj").write_text(obj)
    (tmp_path / "quad.obj").write_text(QUAD)
    scene = TEX_SCENE.replace("tex.obj", "edge.obj").replace("MATERIAL", '<material type="default"/>')
    (tmp_path / "scene.xml").write_text(scene)
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    mats = sc.export("materials").reshape(-1, 16)
    assert mats.shape[0] == 2 and np.allclose(mats[:, :3], 0.6)  # one slot per instance
    assert (sc.export("mat_tex") >> 16).tolist() == [-1] * 4
    uv = sc.export("texcoords").reshape(-1, 2)
    assert {tuple(x) for x in uv.tolist()} == {(0.25, 1.0), (0.5, 0.5)}
    sc.close()
    (tmp_path / "edge.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/x 2 3\n")
    with pytest.raises(ZglError) as e:
        Scene.load(tmp_path / "scene.xml", host_only=True)
    assert e.value.status == 5


def test_crlf_line_endings(zgl_lib, tmp_path):
    """OBJ and MTL files with Windows line endings load like LF ones."""
    _write_textured(tmp_path)
    ref = Scene.load(tmp_path / "scene.xml", host_only=True)
    want = {k: ref.export(k) for k in ("vertices", "texcoords", "mat_tex", "materials", "tex_scale")}
    ref.close()
    for name in ("tex.obj", "tex.mtl"):
        text = (tmp_path / name).read_text()
        (tmp_path / name).write_bytes(text.replace("\n", "\r\n").encode())
    sc = Scene.load(tmp_path / "scene.xml", host_only=True)
    for k, v in want.items():
        assert np.array_equal(sc.export(k), v), k
    sc.close()
