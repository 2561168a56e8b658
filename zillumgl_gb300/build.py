"""Build recipe of libzgl.so (CUDA kernels for sm_103a + C++ host + C ABI).

Every translation unit is compiled by nvcc in parallel and linked into
``zillumgl_gb300/_build/libzgl.so``.  The whole library is compiled without
fused multiply-add (``-fmad=false``, ``-ffp-contract=off`` on the host side)
and with IEEE division and square root, because hit distances and radiance
must be bit-identical to a float32 evaluation of the reference formulas.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libzgl.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-lineinfo",
    "-O3",
    "-std=c++17",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-O2,-Wall,-Wno-unused-function",
    f"-I{INCLUDE}",
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libzgl")
    return path


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every translation unit and link libzgl.so; returns its path."""
    srcs = sources()
    hdrs = headers()
    if not force and not _stale(LIB, srcs + hdrs + [Path(__file__)]):
        return LIB
    objdir = BUILD / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    exe = nvcc()

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.name + ".o")
        cmd = [exe, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cu":
            cmd += ["-Xptxas", "-warn-spills"]
        if verbose:
            print(" ".join(cmd), flush=True)
        _run(cmd)
        return obj

    n = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=n) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    _run([exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
