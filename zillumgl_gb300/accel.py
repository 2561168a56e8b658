"""Accelerator interface: the MTBVH build and its device traversal.

Mirrors the reference's ``BVH(vertices, indices).build() -> PackedBVH``
(src/accelerator/BVH.h:13-47) and the device-side queries ``bvhHit`` /
``bvhTest`` (src/shader/intersection.glsl:367-427).  ``BVH.build()`` builds the
tree on the host and uploads the six threaded tables in the device layout;
the returned :class:`Accelerator` owns them.

Arrays may be numpy arrays (host) or torch tensors (host or CUDA).  CUDA
tensors are used in place and the call is asynchronous on the given stream;
host arrays are staged by the library and the call returns when the results
are back.
"""
from __future__ import annotations

import ctypes as C
from typing import NamedTuple

import numpy as np

from ._lib import call, lib

try:  # torch is optional for host-only use
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _is_torch(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


def _ptr(x) -> int:
    if x is None:
        return 0
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor arguments must be contiguous")
        return x.data_ptr()
    if not x.flags["C_CONTIGUOUS"]:
        raise ValueError("array arguments must be C-contiguous")
    return x.ctypes.data


def _stream_handle(stream) -> int:
    if stream is None:
        if torch is not None and torch.cuda.is_available() and torch.cuda.is_initialized():
            return torch.cuda.current_stream().cuda_stream
        return 0
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _like(ref, shape, dtype_np, dtype_torch):
    if _is_torch(ref):
        return torch.empty(shape, dtype=dtype_torch, device=ref.device)
    return np.empty(shape, dtype=dtype_np)


def _check_rays(origins, dirs) -> int:
    n = origins.shape[0]
    if tuple(origins.shape) != (n, 3) or tuple(dirs.shape) != (n, 3):
        raise ValueError("origins and dirs must both have shape (n, 3)")
    for a in (origins, dirs):
        dt = a.dtype
        if (_is_torch(a) and dt != torch.float32) or (not _is_torch(a) and dt != np.float32):
            raise TypeError("origins and dirs must be float32")
    return n


class PackedBVH(NamedTuple):
    """PackedBVH{bounds, hitTable} (src/accelerator/BVH.h:13-17)."""

    bounds: np.ndarray    # float32 (M, 6): pMin.xyz, pMax.xyz
    hitTable: np.ndarray  # int32 (6, M, 3): {node, prim or -1, miss}


class Accelerator:
    """Device-resident MTBVH (owner of a ``zgl_accel`` handle)."""

    def __init__(self, handle: int, n_triangles: int):
        self._h = C.c_void_p(handle)
        self.n_triangles = n_triangles
        n = C.c_size_t()
        call("zgl_accel_node_count", self._h, C.byref(n))
        self.node_count = n.value

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if self._h:
            call("zgl_accel_destroy", self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- reference-layout export -------------------------------------------
    def export(self) -> PackedBVH:
        M = self.node_count
        bounds = np.empty((M, 6), dtype=np.float32)
        hit = np.empty((6, M, 3), dtype=np.int32)
        call("zgl_accel_export", self._h, _ptr(bounds), _ptr(hit))
        return PackedBVH(bounds, hit)

    SCHEDULES = {"auto": 0, "thread_per_ray": 1, "persistent": 2, "prefetch": 3}

    def set_trace_schedule(self, schedule: str) -> None:
        """Select the trace kernel schedule (results are identical)."""
        call("zgl_accel_set_trace_schedule", self._h, self.SCHEDULES[schedule])

    # -- queries -------------------------------------------------------------
    def trace_closest(self, origins, dirs, hit_id=None, hit_t=None, stream=None):
        """bvhHit: closest primitive id (-1 on miss) and distance (1e8 on miss)."""
        n = _check_rays(origins, dirs)
        if hit_id is None:
            hit_id = _like(origins, (n,), np.int32, torch.int32 if torch else None)
        if hit_t is None:
            hit_t = _like(origins, (n,), np.float32, torch.float32 if torch else None)
        call("zgl_trace_closest", self._h, _ptr(origins), _ptr(dirs), n, _ptr(hit_id), _ptr(hit_t),
             _stream_handle(stream))
        return hit_id, hit_t

    def trace_closest_noalloc(self, origins, dirs, hit_id=None, hit_t=None, stream=None):
        """bvhHit through the allocation-free entry point (at most 262144 rays;
        the library allocates no device memory for the call)."""
        n = _check_rays(origins, dirs)
        if hit_id is None:
            hit_id = _like(origins, (n,), np.int32, torch.int32 if torch else None)
        if hit_t is None:
            hit_t = _like(origins, (n,), np.float32, torch.float32 if torch else None)
        call("zgl_trace_closest_noalloc", self._h, _ptr(origins), _ptr(dirs), n, _ptr(hit_id), _ptr(hit_t),
             _stream_handle(stream))
        return hit_id, hit_t

    def trace_any(self, origins, dirs, tmax, occluded=None, stream=None):
        """bvhTest: 1 where some triangle lies at 0 < t < tmax."""
        n = _check_rays(origins, dirs)
        if occluded is None:
            occluded = _like(origins, (n,), np.uint8, torch.uint8 if torch else None)
        call("zgl_trace_any", self._h, _ptr(origins), _ptr(dirs), _ptr(tmax), n, _ptr(occluded),
             _stream_handle(stream))
        return occluded

    def trace_count(self, origins, dirs, tmax=None, any_hit=False, stream=None):
        """Per-ray table entries visited and triangles tested."""
        n = _check_rays(origins, dirs)
        visits = _like(origins, (n,), np.int32, torch.int32 if torch else None)
        tests = _like(origins, (n,), np.int32, torch.int32 if torch else None)
        call("zgl_trace_count", self._h, _ptr(origins), _ptr(dirs), _ptr(tmax), n, int(bool(any_hit)),
             _ptr(visits), _ptr(tests), _stream_handle(stream))
        return visits, tests


class BVH:
    """``BVH(vertices, indices).build()`` (src/accelerator/BVH.h:26-47).

    ``build()`` constructs the tree on the host, ``build_device()`` with CUDA
    kernels; both give the identical PackedBVH.  Vertices and indices may be
    numpy arrays or (for ``build_device``) CUDA tensors: float32 (n, 3) and
    int32/uint32 (m*3,)."""

    def __init__(self, vertices, indices):
        if _is_torch(vertices) and vertices.is_cuda:
            self._dev = (vertices.reshape(-1, 3).contiguous(), indices.reshape(-1).contiguous())
            index_types = {torch.int32, getattr(torch, "uint32", torch.int32)}
            if self._dev[0].dtype != torch.float32 or self._dev[1].dtype not in index_types:
                raise ValueError("device vertices must be float32 and indices int32/uint32")
            if self._dev[1].numel() % 3:
                raise ValueError("indices must hold 3 entries per triangle")
            self._vertices = None
            self._indices = None
            return
        self._dev = None
        self._vertices = np.ascontiguousarray(np.asarray(vertices, dtype=np.float32).reshape(-1, 3))
        self._indices = np.ascontiguousarray(np.asarray(indices, dtype=np.uint32).reshape(-1))
        if self._indices.size % 3:
            raise ValueError("indices must hold 3 entries per triangle")

    @property
    def vertices(self) -> np.ndarray:
        if self._vertices is None:
            self._vertices = self._dev[0].cpu().numpy()
        return self._vertices

    @property
    def indices(self) -> np.ndarray:
        if self._indices is None:
            self._indices = self._dev[1].cpu().numpy().view(np.uint32)
        return self._indices

    def build_device(self, small_threshold: int = 0, stream=None) -> Accelerator:
        """The accelerator built by CUDA kernels on the current device
        (zgl_accel_build_device); bit-identical to ``build()``."""
        h = C.c_void_p()
        lib()
        v, idx = self._dev if self._dev is not None else (self._vertices, self._indices)
        nv = v.shape[0]
        ntri = (idx.numel() if _is_torch(idx) else idx.size) // 3
        call("zgl_accel_build_device", _ptr(v), nv, _ptr(idx), ntri, int(small_threshold),
             _stream_handle(stream), C.byref(h))
        return Accelerator(h.value, ntri)

    def build_host(self) -> PackedBVH:
        """The PackedBVH built on the host only (no device upload)."""
        ntri = self.indices.size // 3
        M = max(2 * ntri - 1, 0)
        bounds = np.empty((M, 6), dtype=np.float32)
        hit = np.empty((6, M, 3), dtype=np.int32)
        call("zgl_bvh_build_host", _ptr(self.vertices), self.vertices.shape[0], _ptr(self.indices), ntri,
             _ptr(bounds), _ptr(hit))
        return PackedBVH(bounds, hit)

    def build(self) -> Accelerator:
        h = C.c_void_p()
        ntri = self.indices.size // 3
        lib()
        call("zgl_accel_build", _ptr(self.vertices), self.vertices.shape[0], _ptr(self.indices), ntri,
             C.byref(h))
        return Accelerator(h.value, ntri)
