"""Build recipe of the CPU oracle (TEST INFRASTRUCTURE ONLY).

* ``oracle/_build/liborc.so`` — the C++ restatement of the reference hot path
  (compiled with ``-ffp-contract=off`` so that no multiply-add is fused).
* ``oracle/_ref/libzglref.so`` — the reference's own standalone headers
  (``src/math/AliasTable.h``, ``src/math/SobolMatrices256x32.h``) compiled
  from where they lie in the reference tree, when that tree is present.  It is
  built only in the development container and never committed.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
BUILD = ORACLE / "_build"
REF_OUT = ORACLE / "_ref"
LIB = BUILD / "liborc.so"
REF_LIB = REF_OUT / "libzglref.so"
REFERENCE_SRC = Path("/root/reference/src")

CXX = os.environ.get("CXX", "g++")
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
         "-Wall", "-Wdouble-promotion"]


def _sources() -> list[Path]:
    return sorted(p for p in ORACLE.glob("*.cpp") if p.name != "ref_shim.cpp")


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


def build_reference(force: bool = False) -> Path | None:
    """Compile the reference's standalone headers; None when the tree is absent."""
    if not REFERENCE_SRC.is_dir():
        return None
    shim = ORACLE / "ref_shim.cpp"
    if force or _stale(REF_LIB, [shim, Path(__file__)]):
        REF_OUT.mkdir(parents=True, exist_ok=True)
        tmp = REF_LIB.with_suffix(".so.tmp")
        _run([CXX, *FLAGS, f"-I{REFERENCE_SRC}", str(shim), "-o", str(tmp)])
        os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
