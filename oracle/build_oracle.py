"""Build recipe of the CPU oracle and of the reference-code checkers (TEST
INFRASTRUCTURE ONLY).

* ``oracle/_build/liborc.so`` — the C++ restatement of the reference hot path
  (compiled with ``-ffp-contract=off`` so that no multiply-add is fused).
* ``oracle/_ref/libzglref.so`` — the reference's own code, built from the
  reference tree when it is present (the development container; never
  committed, never on the product path):
  - the standalone headers ``src/math/AliasTable.h`` and
    ``src/math/SobolMatrices256x32.h``, compiled where they lie;
  - the MTBVH builder ``src/accelerator/{BVH,AABB}.{h,cpp}`` with
    ``src/util/{Error,Timer,NamespaceDecl}.h``, copied unchanged into
    ``oracle/_ref/src/`` beside the stand-in headers of ``oracle/refstub/``
    (glm, ``core/Buffer.h``, ``core/Model.h``), because ``BVH.h`` includes
    OpenGL and assimp headers through ``../core/`` that cannot exist here.
* ``oracle/_ref/libglslref.so`` — the reference's path-tracer compute shader
  (``src/shader/path_integ_naive.glsl`` and the libraries it includes),
  assembled by the reference's own ``@include`` rule and turned into C++ by
  the mechanical transform of ``oracle/glsl_to_cpp.py``, compiled against
  ``oracle/glsl_shim.h`` and driven by ``oracle/glsl_ref_api.cpp``.

The reference tree is read from ``$ZGL_REFERENCE_TREE`` (default: the
development container's checkout).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
BUILD = ORACLE / "_build"
REF_OUT = ORACLE / "_ref"
LIB = BUILD / "liborc.so"
REF_LIB = REF_OUT / "libzglref.so"
GLSL_LIB = REF_OUT / "libglslref.so"
REFERENCE_TREE = Path(os.environ.get("ZGL_REFERENCE_TREE", "/root/reference"))
REFERENCE_SRC = REFERENCE_TREE / "src"

CXX = os.environ.get("CXX", "g++")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
         "-Wall", "-Wdouble-promotion"]
# the reference's own files are compiled as they are: no warnings are ours to fix there
REF_FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread", "-w"]

# reference files copied unchanged for the MTBVH builder
REF_BVH_FILES = ["accelerator/BVH.h", "accelerator/BVH.cpp", "accelerator/AABB.h", "accelerator/AABB.cpp",
                 "util/Error.h", "util/Timer.h", "util/NamespaceDecl.h"]


def _sources() -> list[Path]:
    """The oracle restatement (files that need the reference tree excluded)."""
    return sorted(p for p in ORACLE.glob("*.cpp") if not p.name.startswith(("ref_", "glsl_")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_oracle(force: bool = False) -> Path:
    srcs = _sources()
    deps = srcs + sorted(ORACLE.glob("*.h")) + [Path(__file__)]
    if force or _stale(LIB, deps):
        BUILD.mkdir(parents=True, exist_ok=True)
        tmp = LIB.with_suffix(".so.tmp")
        _run([CXX, *FLAGS, *map(str, srcs), "-o", str(tmp)])
        os.replace(tmp, LIB)
    return LIB


def _copy_reference_bvh() -> Path:
    """Reference builder sources + stand-in headers under oracle/_ref/src/."""
    dst = REF_OUT / "src"
    for rel in REF_BVH_FILES:
        out = dst / rel
        out.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(REFERENCE_SRC / rel, out)
    stub = ORACLE / "refstub"
    for f in stub.rglob("*"):
        if f.is_file():
            out = dst / f.relative_to(stub)
            out.parent.mkdir(parents=True, exist_ok=True)
            shutil.copyfile(f, out)
    return dst


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference's standalone headers and its MTBVH builder; None
    when the reference tree is absent."""
    if not REFERENCE_SRC.is_dir():
        return None
    shims = [ORACLE / "ref_shim.cpp", ORACLE / "ref_bvh_shim.cpp"]
    stubs = [f for f in (ORACLE / "refstub").rglob("*") if f.is_file()]
    refs = [REFERENCE_SRC / r for r in REF_BVH_FILES]
    if force or _stale(REF_LIB, shims + stubs + refs + [Path(__file__)]):
        REF_OUT.mkdir(parents=True, exist_ok=True)
        src = _copy_reference_bvh()
        tmp = REF_LIB.with_suffix(".so.tmp")
        _run([CXX, *REF_FLAGS, f"-I{src}", f"-I{REFERENCE_SRC}", str(shims[0]), str(shims[1]),
              str(src / "accelerator" / "BVH.cpp"), str(src / "accelerator" / "AABB.cpp"), "-o", str(tmp)])
        os.replace(tmp, REF_LIB)
    return REF_LIB


def build_glsl_reference(force: bool = False) -> Path | None:
    """Transform the reference's path-tracer shader to C++ and compile it; None
    when the reference tree is absent."""
    shader_dir = REFERENCE_SRC / "shader"
    if not shader_dir.is_dir():
        return None
    from .glsl_to_cpp import SHADERS, transform_program

    deps = [ORACLE / "glsl_to_cpp.py", ORACLE / "glsl_shim.h", ORACLE / "glsl_ref_api.cpp", ORACLE / "oracle_math.h",
            ORACLE / "oracle_transc.h", Path(__file__)] + sorted(shader_dir.glob("*.glsl"))
    if force or _stale(GLSL_LIB, deps):
        out = REF_OUT / "glsl"
        out.mkdir(parents=True, exist_ok=True)
        for name, entry in SHADERS.items():
            (out / f"{name}.inc").write_text(transform_program(shader_dir, entry))
        tmp = GLSL_LIB.with_suffix(".so.tmp")
        _run([CXX, *REF_FLAGS, f"-I{ORACLE}", f"-I{out}", str(ORACLE / "glsl_ref_api.cpp"), "-o", str(tmp)])
        os.replace(tmp, GLSL_LIB)
    return GLSL_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
    print(build_glsl_reference(force=True))
