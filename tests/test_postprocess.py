"""The display pass (post_proc.glsl): oracle known answers and image writers
on the CPU, the CUDA kernel bit for bit against the oracle on the GPU."""
from __future__ import annotations

import struct
import zlib

import numpy as np
import pytest

import oracle


def test_oracle_known_answers():
    f = np.array([[[0.0, 0.5, 1.0, 0.0], [2.0, -1.0, np.nan, 0.0]]], np.float32)
    none = oracle.postprocess(f, 2, 1, 1, 1.0, 0)
    assert none[0, 0, 0] == 0.0 and none[0, 0, 2] == 1.0
    assert abs(none[0, 0, 1] - 0.5 ** (1 / 2.2)) < 3e-7
    assert none[0, 1, 1] == 0.0 and none[0, 1, 2] == 0.0  # clamp sends negatives and NaN to 0
    assert np.all(none[..., 3] == 1.0)
    aces = oracle.postprocess(f, 2, 1, 1, 1.0, 2)
    assert abs(aces[0, 0, 2] - (2.54 / 3.16) ** (1 / 2.2)) < 1e-6
    # filmic maps the white point 11.2 / 1.6 to 1
    w = np.full((1, 1, 4), 7.0, np.float32)
    assert abs(oracle.postprocess(w, 1, 1, 1, 1.0, 1)[0, 0, 0] - 1.0) < 1e-6
    # result scale and preview: 4x4 output from a 2x2 film, texel (x // 2, y // 2)
    p = np.arange(16, dtype=np.float32).reshape(2, 2, 4) / 16
    out = oracle.postprocess(p, 4, 4, 2, 0.5, 0)
    assert np.array_equal(out[3, 3], out[2, 2]) and np.array_equal(out[0, 1], out[1, 0])
    assert abs(out[2, 0, 0] - (p[1, 0, 0] * 0.5) ** (1 / 2.2)) < 1e-6
    # a 5-wide output from a 2-wide preview film: column 4 reads past the film -> 0
    out5 = oracle.postprocess(p, 5, 4, 2, 1.0, 0)
    assert np.all(out5[:, 4, :3] == 0.0)


def test_write_pfm_and_png(tmp_path):
    from zillumgl_gb300.image import write_pfm, write_png

    rgb = np.random.default_rng(3).random((5, 7, 3)).astype(np.float32)
    write_pfm(tmp_path / "a.pfm", rgb)
    data = (tmp_path / "a.pfm").read_bytes()
    header = b"PF\n7 5\n-1.0\n"
    assert data.startswith(header)
    back = np.frombuffer(data[len(header):], "<f4").reshape(5, 7, 3)[::-1]
    assert np.array_equal(back, rgb)
    write_png(tmp_path / "a.png", rgb)
    png = (tmp_path / "a.png").read_bytes()
    assert png[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", png[16:24])
    assert (w, h) == (7, 5)
    n = struct.unpack(">I", png[33:37])[0]
    raw = zlib.decompress(png[41:41 + n])
    px = np.frombuffer(raw, np.uint8).reshape(5, 1 + 21)[:, 1:].reshape(5, 7, 3)
    assert np.array_equal(px, np.clip(np.rint(rgb * 255), 0, 255).astype(np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("mapper", [0, 1, 2])
@pytest.mark.parametrize("shape", [(37, 23, 1), (40, 24, 3)])
def test_gpu_postprocess_bit_exact(zgl_lib, cuda, mapper, shape):
    import torch

    from zillumgl_gb300.image import postprocess

    W, H, s = shape
    rng = np.random.default_rng(mapper + 10 * s)
    f = (rng.standard_normal((H // s, W // s, 4)) * 3).astype(np.float32) ** 2
    f[0, 0, 0] = np.nan
    f[0, 1, 1] = np.inf
    f[1, 0, 2] = -5.0
    f[1, 1, 0] = 1e38
    got = postprocess(torch.from_numpy(f).to(cuda), W, H, 0.37, mapper, preview_scale=s).cpu().numpy()
    ref = oracle.postprocess(f, W, H, s, np.float32(0.37), mapper)
    # filmic and ACES turn the clamped 1e30 into inf / inf = NaN; NaN payloads
    # differ between the GPU and the host, so NaNs are compared by position
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))
