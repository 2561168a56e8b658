"""A compiled C++ caller of the integrator ABI (tests/host/naive_path_host.cpp).

The program restates the reference's Integrator interface
(src/core/Integrator.h:25-52) as a thin class over zgl_integrator_*, the way
a NaivePathIntegrator replacement would (src/integrator/NaivePath.cpp:77-115):
it loads a scene XML with zgl_scene_load_xml, renders passes, requests a reset
that the next renderOnePass performs, renders more passes and writes the
frame, sample count and result scale.

* CPU: the program compiles against include/zgl.h and links against libzgl.so.
* GPU: its output equals, bit for bit, the same sequence driven through the
  Python binding (whose frames are checked against the oracle elsewhere).
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "host" / "naive_path_host.cpp"


def _build(zgl_lib, out: Path) -> Path:
    from zillumgl_gb300.build import LIB

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = out / "naive_path_host"
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(SRC),
           f"-L{LIB.parent}", "-lzgl", f"-Wl,-rpath,{LIB.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_host_program_compiles_and_links(zgl_lib, tmp_path):
    exe = _build(zgl_lib, tmp_path)
    assert exe.exists()


@pytest.mark.gpu
def test_host_program_renders_like_the_python_binding(zgl_lib, cuda, tmp_path):
    from tests.test_xml_scene import _write
    from zillumgl_gb300.scene import PathIntegrator, Scene

    exe = _build(zgl_lib, tmp_path)
    _write(tmp_path)
    out = tmp_path / "frame.bin"
    r = subprocess.run([str(exe), str(tmp_path / "scene.xml"), "3", "2", "4", str(out)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    W, H, spp = np.frombuffer(raw[:12], np.int32)
    scale = np.frombuffer(raw[12:16], np.float32)[0]
    frame = np.frombuffer(raw[16:], np.float32).reshape(H, W, 4)

    sc = Scene.load(tmp_path / "scene.xml")
    integ = PathIntegrator(sc, max_depth=4)
    for _ in range(3):
        integ.render_one_pass()
    integ.reset()
    for _ in range(2):
        integ.render_one_pass()
    ref, ref_spp = integ.get_frame()
    assert (W, H) == sc.film and spp == ref_spp == 2
    assert scale == np.float32(integ.result_scale())
    assert np.array_equal(frame.view(np.uint32), ref.view(np.uint32))
    assert frame[..., :3].mean() > 0.0
    integ.close()
    sc.close()
