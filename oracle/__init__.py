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

from .build_oracle import GLSL_LIB, LIB, REF_LIB, REFERENCE_SRC, build_glsl_reference, build_oracle, build_reference

_lib = None
_ref = None
_glsl = None


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
        path = build_reference() if REFERENCE_SRC.is_dir() else (REF_LIB if REF_LIB.exists() else None)
        if path is None or not Path(path).exists():
            return None
        L = C.CDLL(str(path))
        L.ref_alias_build.restype = C.c_int32
        L.ref_alias_build.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.ref_sobol_matrices.restype = C.c_int32
        L.ref_sobol_matrices.argtypes = [C.c_void_p, C.c_int32]
        L.ref_bvh_build.restype = C.c_int64
        L.ref_bvh_build.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        _ref = L
    return _ref


def glsl_lib() -> C.CDLL | None:
    """The reference's path-tracer shader compiled as C++ (oracle/glsl_to_cpp.py),
    or None without the reference tree."""
    global _glsl
    if _glsl is None:
        path = build_glsl_reference() if REFERENCE_SRC.is_dir() else (GLSL_LIB if GLSL_LIB.exists() else None)
        if path is None or not Path(path).exists():
            return None
        L = C.CDLL(str(path))
        L.glslref_render_pt.restype = None
        L.glslref_render_pt.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_int32]
        L.glslref_render_lt.restype = None
        L.glslref_render_lt.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
        L.glslref_render_triple.restype = None
        L.glslref_render_triple.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                            C.c_void_p, C.c_int32]
        L.glslref_trace.restype = None
        L.glslref_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                    C.c_void_p, C.c_int32]
        _glsl = L
    return _glsl


def glsl_trace(packed_bounds, packed_hit, vertices, indices, origins, dirs, tmax=None, nthreads=None):
    """bvhHit / bvhTest of the reference shader source (compiled as C++) on a
    PackedBVH: (hit id or occluded flag, distance), or None without the
    reference tree."""
    L = glsl_lib()
    if L is None:
        return None
    b = np.ascontiguousarray(packed_bounds, np.float32)
    h = np.ascontiguousarray(packed_hit, np.int32)
    v = np.ascontiguousarray(vertices, np.float32)
    idx = np.ascontiguousarray(indices, np.uint32)
    s = OrcScene()
    s.vertices, s.normals, s.indices = _p(v), _p(v), _p(idx)
    s.nTriangles = s.objPrimCount = idx.size // 3
    s.bounds, s.hitTable, s.bvhSize = _p(b), _p(h), b.shape[0]
    o = np.ascontiguousarray(origins, np.float32)
    d = np.ascontiguousarray(dirs, np.float32)
    tm = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
    hit = np.zeros(o.shape[0], np.int32)
    dist = np.zeros(o.shape[0], np.float32)
    L.glslref_trace(C.addressof(s), _p(o), _p(d), _p(tm), o.shape[0], _p(hit), _p(dist), nthreads or threads())
    return hit, dist


def ref_bvh_build(vertices: np.ndarray, indices: np.ndarray):
    """PackedBVH of the reference's own BVH::build() (src/accelerator/BVH.cpp,
    compiled from the reference tree): (bounds (M,6) f32, hitTable (6,M,3)
    i32), or None without the reference tree.  The mesh must not be empty."""
    ref = ref_lib()
    if ref is None:
        return None
    v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
    ntri = idx.size // 3
    if ntri == 0:
        raise ValueError("the reference builder does not handle an empty mesh")
    M = 2 * ntri - 1
    bounds = np.zeros((M, 6), np.float32)
    hit = np.zeros((6, M, 3), np.int32)
    r = ref.ref_bvh_build(_p(v), v.shape[0], _p(idx), ntri, _p(bounds), _p(hit))
    assert r == M
    return bounds, hit


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


# ---------------------------------------------------------------------------
# Path tracer oracle
# ---------------------------------------------------------------------------
class OrcScene(C.Structure):
    _fields_ = [
        ("vertices", C.c_void_p), ("normals", C.c_void_p), ("indices", C.c_void_p), ("matTexIndex", C.c_void_p),
        ("nTriangles", C.c_int64), ("objPrimCount", C.c_int32),
        ("bounds", C.c_void_p), ("hitTable", C.c_void_p), ("bvhSize", C.c_int64),
        ("materials", C.c_void_p),
        ("nLightTriangles", C.c_int32), ("lightPower", C.c_void_p), ("lightAlias", C.c_void_p),
        ("lightProb", C.c_void_p), ("lightSum", C.c_float),
        ("envTexels", C.c_void_p), ("envWidth", C.c_int32), ("envHeight", C.c_int32), ("envAlias", C.c_void_p),
        ("envProb", C.c_void_p), ("envSum", C.c_float), ("envRotation", C.c_float),
        ("sobolMatrices", C.c_void_p), ("noise", C.c_void_p), ("sampler", C.c_int32),
        ("camF", C.c_float * 3), ("camR", C.c_float * 3), ("camU", C.c_float * 3), ("camPos", C.c_float * 3),
        ("camMatInv", C.c_float * 9), ("tanFOV", C.c_float), ("lensRadius", C.c_float), ("focalDist", C.c_float),
        ("camAsp", C.c_float), ("filmW", C.c_int32), ("filmH", C.c_int32),
        ("maxDepth", C.c_int32), ("russianRoulette", C.c_int32), ("sampleLight", C.c_int32),
        ("lightEnvUniformSample", C.c_int32), ("lightPortion", C.c_float), ("rrStartDepth", C.c_int32),
        ("texCoords", C.c_void_p), ("nTextures", C.c_int32), ("texMaxW", C.c_int32), ("texMaxH", C.c_int32),
        ("texLayers", C.c_void_p), ("texScale", C.c_void_p),
    ]


def texture_layers(textures):
    """Texture2DArray (Texture.cpp:134-171): (layers uint8 (n, Hmax, Wmax, 3)
    with each image in the top-left corner, uv scales float32 (n, 2))."""
    if not textures:
        return None, None
    wmax = max(t.shape[1] for t in textures)
    hmax = max(t.shape[0] for t in textures)
    layers = np.zeros((len(textures), hmax, wmax, 3), np.uint8)
    scale = np.zeros((len(textures), 2), np.float32)
    for k, t in enumerate(textures):
        layers[k, :t.shape[0], :t.shape[1]] = t
        scale[k] = (np.float32(t.shape[1]) / np.float32(wmax), np.float32(t.shape[0]) / np.float32(hmax))
    return layers, scale


def _render_lib():
    L = lib()
    if not getattr(L, "_render_ready", False):
        L.orc_light_tables.restype = C.c_float
        L.orc_light_tables.argtypes = [C.c_void_p] * 4 + [C.c_int32] + [C.c_void_p] * 3
        L.orc_env_tables.restype = C.c_float
        L.orc_env_tables.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
        L.orc_noise.restype = None
        L.orc_noise.argtypes = [C.c_int32, C.c_int32, C.c_void_p]
        L.orc_camera.restype = None
        L.orc_camera.argtypes = [C.c_void_p, C.c_float, C.c_void_p]
        L.orc_render_pt.restype = None
        L.orc_render_pt.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                    C.c_void_p, C.c_int32]
        L.orc_render_pt_frozen.restype = None
        L.orc_render_pt_frozen.argtypes = [C.POINTER(OrcScene), C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                           C.c_void_p, C.c_int64, C.c_void_p, C.c_int32]
        L.orc_render_lt.restype = None
        L.orc_render_lt.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
        L.orc_render_triple.restype = None
        L.orc_render_triple.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                        C.c_void_p]
        L.orc_render_mt.restype = None
        L.orc_render_mt.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_void_p, C.c_int32]
        L.orc_alias_build.restype = None
        L.orc_alias_build.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
        L.orc_transc.restype = None
        L.orc_transc.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_postprocess.restype = None
        L.orc_postprocess.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_int32, C.c_void_p]
        L.orc_texture_sample.restype = None
        L.orc_texture_sample.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]
        L.orc_diff_grad.restype = None
        L.orc_diff_grad.argtypes = [C.POINTER(OrcScene), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                    C.c_int32, C.c_void_p, C.c_int32]
        L._render_ready = True
    return L


def light_tables(data):
    """(lightPower (nL,3), alias, prob, lightSum) restating Scene.cpp:200-243."""
    nl = data.light_indices.size // 3
    power = np.zeros((nl, 3), np.float32)
    alias = np.zeros(nl, np.int32)
    prob = np.zeros(nl, np.float32)
    if nl == 0:
        return power, alias, prob, np.float32(0)
    s = _render_lib().orc_light_tables(_p(data.light_vertices), _p(data.light_indices), _p(data.light_first),
                                       _p(data.light_power), data.light_power.shape[0], _p(power), _p(alias),
                                       _p(prob))
    return power, alias, prob, np.float32(s)


def alias_build(pdf):
    pdf = np.ascontiguousarray(pdf, np.float32)
    alias = np.zeros(pdf.size, np.int32)
    prob = np.zeros(pdf.size, np.float32)
    _render_lib().orc_alias_build(_p(pdf), pdf.size, _p(alias), _p(prob))
    return alias, prob


def ref_alias_build(pdf):
    """AliasTable::build from the reference header itself (None without the tree)."""
    ref = ref_lib()
    if ref is None:
        return None
    pdf = np.ascontiguousarray(pdf, np.float32)
    alias = np.zeros(pdf.size, np.int32)
    prob = np.zeros(pdf.size, np.float32)
    ref.ref_alias_build(_p(pdf), pdf.size, _p(alias), _p(prob))
    return alias, prob


def env_tables(rgb):
    """(alias, prob, sum) restating EnvironmentMap.cpp:8-114 for an (H, W, 3) image."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    H, W = rgb.shape[:2]
    alias = np.zeros((W + 1) * H, np.int32)
    prob = np.zeros((W + 1) * H, np.float32)
    s = _render_lib().orc_env_tables(_p(rgb), W, H, _p(alias), _p(prob))
    return alias, prob, np.float32(s)


def noise(W, H):
    out = np.zeros(W * H * 2, np.float32)
    _render_lib().orc_noise(W, H, _p(out))
    return out


def camera(angle, fov):
    out = np.zeros(19, np.float32)
    a = np.ascontiguousarray(angle, np.float32)
    _render_lib().orc_camera(_p(a), float(min(max(fov, 0.1), 90.0)), _p(out))
    return out


def postprocess(frame, width, height, preview_scale, result_scale, tone_mapper):
    """post_proc.glsl's display pass on a (H/s, W/s, 4) RGBA sum -> (H, W, 4)."""
    frame = np.ascontiguousarray(frame, np.float32)
    out = np.zeros((height, width, 4), np.float32)
    _render_lib().orc_postprocess(_p(frame), width, height, preview_scale, float(result_scale), tone_mapper, _p(out))
    return out


def transc(op, a, b=None):
    a = np.ascontiguousarray(a, np.float32)
    out = np.empty_like(a)
    bb = None if b is None else np.ascontiguousarray(b, np.float32)
    _render_lib().orc_transc(op, _p(a), _p(bb), _p(out), a.size)
    return out


class OracleScene:
    """The oracle's own flattening, BVH and tables for a SceneData; the Sobol
    matrices are an input (checked against the reference table separately)."""

    def __init__(self, data, sobol_matrices, params=None):
        v, n, idx = data.flat()
        self.v, self.n, self.idx = v, n, idx
        self.bounds, self.hit, _ = bvh_build(v, idx)
        self.mat_tex = np.ascontiguousarray(data.obj_mat_tex, np.int32)
        self.materials = np.ascontiguousarray(data.materials, np.float32)
        self.light_power, self.light_alias, self.light_prob, self.light_sum = light_tables(data)
        self.sobol = np.ascontiguousarray(sobol_matrices, np.uint32)
        W, H = data.film
        self.noise = noise(W, H)
        self.cam = camera(data.cam_angle, data.cam_fov)
        s = OrcScene()
        s.vertices, s.normals, s.indices, s.matTexIndex = _p(v), _p(n), _p(idx), _p(self.mat_tex)
        s.nTriangles = idx.size // 3
        s.objPrimCount = data.obj_indices.size // 3
        s.bounds, s.hitTable, s.bvhSize = _p(self.bounds), _p(self.hit), self.bounds.shape[0]
        s.materials = _p(self.materials)
        s.nLightTriangles = data.light_indices.size // 3
        s.lightPower, s.lightAlias, s.lightProb = _p(self.light_power), _p(self.light_alias), _p(self.light_prob)
        s.lightSum = float(self.light_sum)
        if data.env_rgb is not None:
            rgb = np.ascontiguousarray(data.env_rgb, np.float32)
            self.env_texels = rgb.astype(np.float16).astype(np.float32).reshape(-1)
            self.env_alias, self.env_prob, esum = env_tables(rgb)
            s.envTexels, s.envAlias, s.envProb = _p(self.env_texels), _p(self.env_alias), _p(self.env_prob)
            s.envHeight, s.envWidth = rgb.shape[0], rgb.shape[1]
            s.envSum = float(np.float32(int(esum)))
        else:
            s.envTexels = None
            s.envSum = 0.0
        s.envRotation = data.env_rotation
        s.sobolMatrices, s.noise, s.sampler = _p(self.sobol), _p(self.noise), data.sampler
        c = self.cam
        s.camF = (C.c_float * 3)(*c[0:3])
        s.camR = (C.c_float * 3)(*c[3:6])
        s.camU = (C.c_float * 3)(*c[6:9])
        s.camMatInv = (C.c_float * 9)(*c[9:18])
        s.tanFOV = float(c[18])
        s.camPos = (C.c_float * 3)(*data.cam_pos)
        s.lensRadius, s.focalDist = data.cam_lens_radius, data.cam_focal_dist
        s.filmW, s.filmH = W, H
        s.camAsp = float(np.float32(W) / np.float32(H))
        textures = getattr(data, "textures", None)
        if textures:
            self.tex_layers, self.tex_scale = texture_layers(textures)
            tc = getattr(data, "obj_texcoords", None)
            nvo = np.asarray(data.obj_vertices).reshape(-1, 3).shape[0]
            self.texcoords = (np.zeros((nvo, 2), np.float32) if tc is None
                              else np.ascontiguousarray(np.asarray(tc, np.float32).reshape(-1, 2)))
            s.texCoords, s.texLayers, s.texScale = _p(self.texcoords), _p(self.tex_layers), _p(self.tex_scale)
            s.nTextures = len(textures)
            s.texMaxH, s.texMaxW = self.tex_layers.shape[1], self.tex_layers.shape[2]
        p = params or {}
        s.maxDepth = p.get("max_depth", 4)
        s.russianRoulette = p.get("russian_roulette", 0)
        s.sampleLight = p.get("sample_light", 1)
        s.lightEnvUniformSample = p.get("light_env_uniform_sample", 0)
        s.lightPortion = p.get("light_portion", 0.5)
        s.rrStartDepth = p.get("rr_start_depth", 1)
        self.s = s

    def texture_sample(self, tex_id, uv):
        """The albedo texture lookup at texcoords uv (n, 2) -> rgb (n, 3)."""
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        out = np.zeros((uv.shape[0], 3), np.float32)
        _render_lib().orc_texture_sample(C.byref(self.s), int(tex_id), _p(uv), uv.shape[0], _p(out))
        return out

    def render_pt(self, pixels, passes, spp0=0, fc0=1, nthreads=None):
        """Sum of `passes` progressive passes for the pixel indices (y * W + x)."""
        pix = np.ascontiguousarray(pixels, np.int32)
        out = np.zeros((pix.size, 3), np.float32)
        _render_lib().orc_render_pt(C.byref(self.s), spp0, passes, fc0, _p(pix), pix.size, _p(out),
                                    nthreads or threads())
        return out

    def render_pt_frozen(self, materials, pixels, passes, spp0=0, fc0=1, nthreads=None):
        """render_pt with every sampling decision of this scene but the BSDF
        values of `materials` (n, 16): the detached-sampling estimator whose
        finite differences check the adjoint's material gradients."""
        mat = np.ascontiguousarray(materials, np.float32)
        assert mat.size == self.materials.size
        pix = np.ascontiguousarray(pixels, np.int32)
        out = np.zeros((pix.size, 3), np.float32)
        _render_lib().orc_render_pt_frozen(C.byref(self.s), _p(mat), spp0, passes, fc0, _p(pix), pix.size, _p(out),
                                           nthreads or threads())
        return out

    def glsl_render_pt(self, pixels, passes, spp0=0, fc0=1, nthreads=None):
        """render_pt by the reference's own shader source compiled as C++
        (None without the reference tree).  Russian roulette follows the
        shader, which starts it at the first bounce."""
        L = glsl_lib()
        if L is None:
            return None
        pix = np.ascontiguousarray(pixels, np.int32)
        out = np.zeros((pix.size, 3), np.float32)
        L.glslref_render_pt(C.addressof(self.s), spp0, passes, fc0, _p(pix), pix.size, _p(out), nthreads or threads())
        return out

    def glsl_render_lt(self, passes, blocks=32, spp0=0, fc0=1):
        """render_lt by the reference's light_path_integ.glsl compiled as C++."""
        L = glsl_lib()
        if L is None:
            return None
        film = np.zeros((self.s.filmH, self.s.filmW, 3), np.float32)
        L.glslref_render_lt(C.addressof(self.s), spp0, passes, fc0, blocks, _p(film))
        return film

    def glsl_render_triple(self, passes, blocks=64, loops=1, spp0=0, fc0=1, nthreads=None):
        """render_triple by the reference's triple_path_pass_{pt,lpt}.glsl
        compiled as C++."""
        L = glsl_lib()
        if L is None:
            return None
        film = np.zeros((self.s.filmH, self.s.filmW, 3), np.float32)
        L.glslref_render_triple(C.addressof(self.s), spp0, passes, fc0, blocks, loops, _p(film), nthreads or threads())
        return film

    def glsl_trace(self, origins, dirs, tmax=None, nthreads=None):
        """bvhHit (or bvhTest with tmax) of the reference shader on this
        scene's PackedBVH: (hit id or occluded flag, distance)."""
        L = glsl_lib()
        if L is None:
            return None
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(dirs, np.float32)
        tm = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
        hit = np.zeros(o.shape[0], np.int32)
        dist = np.zeros(o.shape[0], np.float32)
        L.glslref_trace(C.addressof(self.s), _p(o), _p(d), _p(tm), o.shape[0], _p(hit), _p(dist), nthreads or threads())
        return hit, dist

    def render_lt(self, passes, blocks=32, spp0=0, fc0=1):
        """Film sum (H, W, 3) of `passes` light-tracer passes."""
        W, H = self.s.filmW, self.s.filmH
        film = np.zeros((H, W, 3), np.float32)
        _render_lib().orc_render_lt(C.byref(self.s), spp0, passes, fc0, blocks, _p(film))
        return film

    def render_triple(self, passes, blocks=64, loops=1, spp0=0, fc0=1):
        """Film sum (H, W, 3) of `passes` triple-integrator passes."""
        W, H = self.s.filmW, self.s.filmH
        film = np.zeros((H, W, 3), np.float32)
        _render_lib().orc_render_triple(C.byref(self.s), spp0, passes, fc0, blocks, loops, _p(film))
        return film

    def render_threaded(self, kind, passes, blocks, loops=1, spp0=0, fc0=1, nthreads=None):
        """Light tracer (kind "light") or triple integrator (kind "triple")
        passes on `nthreads` host threads with per-thread films: the CPU
        baseline's timing path.  Equal to render_lt / render_triple up to the
        order of float additions."""
        W, H = self.s.filmW, self.s.filmH
        film = np.zeros((H, W, 3), np.float32)
        _render_lib().orc_render_mt(C.byref(self.s), 0 if kind == "light" else 1, spp0, passes, fc0, blocks, loops,
                                    _p(film), nthreads or threads())
        return film

    def diff_grad(self, data, spp, dimage, nthreads=None):
        """Gradient oracle of the differentiable renderer: d sum(dimage * mean
        image of samples 0..spp-1) / d (material, light power) parameters, FP64."""
        nmat = data.materials.size // 16
        first = np.asarray(data.light_first, np.int64)
        ninst = max(first.size - 1, 0)
        inst = np.zeros(max(data.light_indices.size // 3, 1), np.int32)
        for k in range(ninst):
            inst[first[k]:first[k + 1]] = k
        power = np.ascontiguousarray(data.light_power, np.float32).reshape(-1)
        if power.size == 0:
            power = np.zeros(1, np.float32)
        dimg = np.ascontiguousarray(dimage, np.float32)
        grad = np.zeros(nmat * 6 + ninst * 3, np.float64)
        _render_lib().orc_diff_grad(C.byref(self.s), spp, _p(dimg), _p(inst), _p(power), nmat, ninst, _p(grad),
                                    nthreads or threads())
        return grad
