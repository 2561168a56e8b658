"""zillumgl_gb300 — GB300-native render hot path of ZillumGL.

CUDA kernels for sm_103a behind a C ABI (include/zgl.h, built into
``_build/libzgl.so``) and a thin Python mirror of the reference's interfaces.
"""
from ._lib import LIB_PATH, ZglError, lib
from .accel import BVH, Accelerator, PackedBVH

__all__ = ["LIB_PATH", "ZglError", "lib", "BVH", "Accelerator", "PackedBVH"]
