"""Display and image output: the reference's tone-mapping pass
(src/shader/post_proc.glsl) on the GPU through zgl_postprocess, and PFM / PNG
writers for its results."""
from __future__ import annotations

import struct
import zlib

import numpy as np

from ._lib import call

TONE_NONE, TONE_FILMIC, TONE_ACES = 0, 1, 2


def postprocess(frame, width: int, height: int, result_scale: float, tone_mapper: int = TONE_FILMIC,
                preview_scale: int = 1, out=None, stream=None):
    """pow(tone(clamp(frame * result_scale, 0, 1e30)), 1/2.2), alpha 1.

    ``frame`` is a CUDA float32 tensor (height // preview_scale,
    width // preview_scale, 4) holding the accumulated sum; returns a CUDA
    float32 tensor (height, width, 4)."""
    import torch

    from .accel import _ptr, _stream_handle

    if out is None:
        out = torch.empty((height, width, 4), dtype=torch.float32, device=frame.device)
    call("zgl_postprocess", _ptr(frame.contiguous()), int(width), int(height), int(preview_scale),
         float(result_scale), int(tone_mapper), _ptr(out), _stream_handle(stream))
    return out


def write_pfm(path, rgb) -> None:
    """Portable float map, little endian, rows bottom to top (as PFM stores them)."""
    rgb = np.ascontiguousarray(np.asarray(rgb, np.float32)[..., :3])
    h, w = rgb.shape[:2]
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(rgb[::-1].astype("<f4").tobytes())


def write_png(path, rgb) -> None:
    """8-bit RGB PNG of values in [0, 1] (rounded, clamped), no filtering."""
    a = np.asarray(rgb, np.float32)[..., :3]
    a = np.clip(np.rint(np.nan_to_num(a) * 255.0), 0, 255).astype(np.uint8)
    h, w = a.shape[:2]
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
