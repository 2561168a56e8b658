"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker of the CUDA path.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import this
package; the product (``zillumgl_gb300``) never does.

Parity: the reference's device code is GLSL and cannot run here, so the
oracle restates it in C++ (parity unpinned at the shader level).  The two
reference headers that compile on their own (``src/math/AliasTable.h``,
``src/math/SobolMatrices256x32.h``) are compiled into ``oracle/_ref/`` in the
development container and pin the tables that depend on them.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from .build_oracle import LIB, REF_LIB, build_oracle, build_reference

_lib = None
_ref = None


def _p(a):
    return None if a is None else a.ctypes.data


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(str(LIB))
        L.orc_bvh_build.restype = C.c_int64
        L.orc_bvh_build.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
        L.orc_trace.restype = None
        L.orc_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_int32]
        _lib = L
    return _lib


def ref_lib() -> C.CDLL | None:
    """The reference's own standalone headers, or None when unavailable."""
    global _ref
    if _ref is None:
        path = build_reference() if Path("/root/reference/src").is_dir() else (REF_LIB if REF_LIB.exists() else None)
        if path is None or not Path(path).exists():
            return None
        L = C.CDLL(str(path))
        L.ref_alias_build.restype = C.c_int32
        L.ref_alias_build.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.ref_sobol_matrices.restype = C.c_int32
        L.ref_sobol_matrices.argtypes = [C.c_void_p, C.c_int32]
        _ref = L
    return _ref


def threads() -> int:
    return max(1, os.cpu_count() or 1)


def bvh_build(vertices: np.ndarray, indices: np.ndarray):
    """PackedBVH of the oracle: (bounds (M,6) f32, hitTable (6,M,3) i32, sizeIndices (M,) i32)."""
    v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
    ntri = idx.size // 3
    M = max(2 * ntri - 1, 0)
    bounds = np.zeros((M, 6), np.float32)
    hit = np.zeros((6, M, 3), np.int32)
    sizes = np.zeros((M,), np.int32)
    r = lib().orc_bvh_build(_p(v), v.shape[0], _p(idx), ntri, _p(bounds), _p(hit), _p(sizes))
    if r < 0:
        raise ValueError("oracle: index out of range")
    return bounds, hit, sizes


def trace(packed_bounds, packed_hit, vertices, indices, origins, dirs, tmax=None, any_hit=False,
          nthreads: int | None = None):
    """Oracle traversal: returns (hit_id or occluded, hit_t, visits, tests)."""
    b = np.ascontiguousarray(packed_bounds, np.float32)
    h = np.ascontiguousarray(packed_hit, np.int32)
    v = np.ascontiguousarray(vertices, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32)
    o = np.ascontiguousarray(origins, np.float32)
    d = np.ascontiguousarray(dirs, np.float32)
    n = o.shape[0]
    tm = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
    if any_hit and tm is None:
        raise ValueError("any-hit traversal needs tmax")
    hid = np.zeros(n, np.int32)
    ht = np.zeros(n, np.float32)
    vis = np.zeros(n, np.int32)
    tst = np.zeros(n, np.int32)
    lib().orc_trace(_p(b), _p(h), b.shape[0], _p(v), _p(idx), _p(o), _p(d), _p(tm), n, int(any_hit), _p(hid),
                    _p(ht), _p(vis), _p(tst), nthreads or threads())
    return hid, ht, vis, tst
