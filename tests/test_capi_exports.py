"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU work)."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:zgl_status|int32_t|const char\*|void)\s+(zgl_\w+)\s*\(", text, flags=re.M)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "zgl_trace_closest" in names and "zgl_accel_build" in names
    assert len(names) == len(set(names))


def test_library_exports_every_declared_symbol(zgl_lib):
    missing = [n for n in declared_symbols() if not hasattr(zgl_lib, n)]
    assert not missing, f"libzgl.so lacks {missing}"


def test_python_binding_covers_header(zgl_lib):
    from zillumgl_gb300._lib import SIGNATURES

    assert set(declared_symbols()) == set(SIGNATURES)


def test_version_and_error_string(zgl_lib):
    assert zgl_lib.zgl_version() >= 100
    assert isinstance(zgl_lib.zgl_last_error(), bytes)


def test_invalid_arguments_return_status_not_abort(zgl_lib):
    from zillumgl_gb300 import BVH, ZglError

    v = np.zeros((3, 3), np.float32)
    with pytest.raises(ZglError) as e:
        BVH(v, np.array([0, 1, 7], np.uint32)).build_host()
    assert e.value.status == 1 and "out of range" in str(e.value)
    bad = v.copy()
    bad[1, 1] = np.nan
    with pytest.raises(ZglError):
        BVH(bad, np.array([0, 1, 2], np.uint32)).build_host()
    # beyond quickBuild's default box (+-1e8) and infinite coordinates
    for x in (2e8, -np.inf):
        bad = v.copy()
        bad[2, 0] = x
        with pytest.raises(ZglError) as e:
            BVH(bad, np.array([0, 1, 2], np.uint32)).build_host()
        assert "1e8" in str(e.value)
    edge = v.copy()
    edge[2] = (1e8, -1e8, 0.5)
    assert BVH(edge, np.array([0, 1, 2], np.uint32)).build_host().bounds.shape == (1, 6)


def test_device_build_argument_checks_need_no_gpu(zgl_lib):
    """zgl_accel_build_device validates its arguments before any device work."""
    import ctypes as C

    from zillumgl_gb300 import BVH, ZglError
    from zillumgl_gb300._lib import call

    v = np.zeros((3, 3), np.float32)
    i = np.array([0, 1, 2], np.uint32)
    for bad in (5000, -1):
        with pytest.raises(ZglError) as e:
            BVH(v, i).build_device(small_threshold=bad)
        assert e.value.status == 1 and "small_threshold" in str(e.value)
    with pytest.raises(ZglError) as e:
        call("zgl_accel_build_device", v.ctypes.data, 3, i.ctypes.data, 1, 0, 0, None)
    assert e.value.status == 1
    with pytest.raises(ZglError) as e:
        out = C.c_void_p()
        call("zgl_accel_build_device", None, 3, None, 1, 0, 0, C.byref(out))
    assert e.value.status == 1


def test_header_is_plain_c99(tmp_path):
    """include/zgl.h compiles as C99 (-pedantic, warnings as errors) in a C
    translation unit that takes the address of every entry point it declares
    (the boundary a C or FFI caller binds)."""
    import re
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = Path(__file__).resolve().parents[1]
    header = (root / "include" / "zgl.h").read_text()
    names = sorted(set(re.findall(r"\b(zgl_[a-z0-9_]+)\s*\(", header)))
    src = tmp_path / "use.c"
    refs = "\n".join(f"    (void)&{n};" for n in names)
    src.write_text(f'#include "zgl.h"\nint main(void) {{\n    zgl_scene_desc d = {{0}};\n    (void)d;\n{refs}\n'
                   "    return 0;\n}\n")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{root / 'include'}", "-c",
                        str(src), "-o", str(tmp_path / "use.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert len(names) > 40
