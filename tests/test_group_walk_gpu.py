"""The integrators' long-ray walk (traverse.cuh: traverse_lane_m +
finish_long_rays_group) under the warp compositions the renderers produce:
lanes of one warp split into divergent groups, so walks run with fewer than
32 lanes, and neighbouring lanes tracing in different accelerators (the
batched renderer's persistent and queue schedules mix requests in a warp).
Rays with a near-zero direction component (boxHit's near-zero branch) that
outrun the lane budget are walked by their group; every hit id, distance and
any-hit flag must equal the oracle's in that ray's own scene
(src/shader/intersection.glsl:367-427).

tests/cuda/group_walk.cu holds the test kernel; it is compiled here from the
product's own traverse.cuh with the product's nvcc flags."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle
from zillumgl_gb300 import BVH
from zillumgl_gb300.synthetic import triangle_soup

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent
SRC = HERE / "cuda" / "group_walk.cu"
OUT = HERE / "cuda" / "_build" / "libgroupwalk.so"


def _library():
    from zillumgl_gb300 import build as B

    deps = [SRC, B.CSRC / "traverse.cuh", B.CSRC / "accel.h"]
    if not OUT.exists() or OUT.stat().st_mtime < max(p.stat().st_mtime for p in deps):
        OUT.parent.mkdir(parents=True, exist_ok=True)
        B._run([B.nvcc(), *B.NVCC_FLAGS, "-shared", f"-I{B.CSRC}", f"-I{B.INCLUDE}", str(SRC), "-o", str(OUT)])
    lib = C.CDLL(str(OUT))
    lib.group_walk.restype = C.c_int
    lib.group_walk.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p]
    return lib


def _device_tables(v, idx, cuda):
    """Node records and traversal triangles laid out as the library keeps them
    (accel.h): per face entry (pMin.xyz, prim) (pMax.xyz, miss); per triangle
    a.xyz ab.x | ab.yz ac.xy | ac.z (float32 differences)."""
    import torch

    acc = BVH(v, idx).build()
    p = acc.export()
    acc.close()
    m = p.bounds.shape[0] // 6 if p.bounds.ndim == 1 else p.bounds.shape[0]
    b = np.asarray(p.bounds, np.float32).reshape(m, 6)
    hit = np.asarray(p.hitTable, np.int32).reshape(6 * m, 3)
    rec = np.zeros((6 * m, 2, 4), np.float32)
    rec[:, 0, :3] = b[hit[:, 0], :3]
    rec[:, 0, 3] = hit[:, 1].copy().view(np.float32)
    rec[:, 1, :3] = b[hit[:, 0], 3:]
    rec[:, 1, 3] = hit[:, 2].copy().view(np.float32)
    tri = idx.reshape(-1, 3)
    a, bb, c = v[tri[:, 0]], v[tri[:, 1]], v[tri[:, 2]]
    ab, ac = bb - a, c - a
    t = np.zeros((tri.shape[0], 3, 4), np.float32)
    t[:, 0, :3], t[:, 0, 3] = a, ab[:, 0]
    t[:, 1, 0], t[:, 1, 1], t[:, 1, 2], t[:, 1, 3] = ab[:, 1], ab[:, 2], ac[:, 0], ac[:, 1]
    t[:, 2, 0] = ac[:, 2]
    return torch.from_numpy(rec).to(cuda), torch.from_numpy(t).to(cuda), m, p


def _rays(rng, n):
    """Every other ray has one direction component below 1e-6 in magnitude
    (long in a dense soup); the rest are random."""
    o = rng.random((n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3))
    long_ = np.arange(n) % 4 < 2
    axis = rng.integers(0, 3, n)
    sel = np.nonzero(long_)[0]
    d[sel, axis[sel]] = rng.choice([-1.0, 1.0], sel.size) * rng.uniform(1e-8, 9e-7, sel.size)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


@pytest.mark.parametrize("any_hit", [False, True])
def test_group_walks_with_divergent_groups_and_mixed_accelerators(zgl_lib, cuda, any_hit):
    import torch

    lib = _library()
    va, ia = triangle_soup(60000, 5)
    vb, ib = triangle_soup(30000, 7)
    na, ta, ma, pa = _device_tables(va, ia, cuda)
    nb, tb, mb, pb = _device_tables(vb, ib, cuda)
    n = 8192 + 77  # a partial last warp as well
    o, d = _rays(np.random.default_rng(51), n)
    tmax = (np.random.default_rng(52).random(n) * 2.0).astype(np.float32)
    even, odd = np.arange(0, n, 2), np.arange(1, n, 2)  # ray i traces in scene A (even) or B (odd)
    ra = oracle.trace(pa.bounds, pa.hitTable, va, ia, o[even], d[even], tmax=tmax[even] if any_hit else None,
                      any_hit=any_hit)
    rb = oracle.trace(pb.bounds, pb.hitTable, vb, ib, o[odd], d[odd], tmax=tmax[odd] if any_hit else None,
                      any_hit=any_hit)
    assert int((ra[2] > 256).sum()) >= 50 and int((rb[2] > 256).sum()) >= 20, "too few rays past the budget"
    to, td, tm = (torch.from_numpy(x).to(cuda) for x in (o, d, tmax))
    out_id = torch.full((n,), -7, dtype=torch.int32, device=cuda)
    out_t = torch.zeros(n, dtype=torch.float32, device=cuda)
    rc = lib.group_walk(na.data_ptr(), ta.data_ptr(), ma, nb.data_ptr(), tb.data_ptr(), mb, to.data_ptr(),
                        td.data_ptr(), tm.data_ptr(), n, int(any_hit), out_id.data_ptr(), out_t.data_ptr())
    assert rc == 0, f"CUDA error {rc}"
    g_id, g_t = out_id.cpu().numpy(), out_t.cpu().numpy()
    for sel, ref in ((even, ra), (odd, rb)):
        assert np.array_equal(g_id[sel], ref[0].astype(np.int32)), "hit ids / flags differ"
        if not any_hit:
            assert np.array_equal(g_t[sel].view(np.uint32), ref[1].view(np.uint32)), "distances differ"
