"""Scene and integrator interfaces.

``Scene`` mirrors ``Scene::createGLContext`` (src/core/Scene.cpp:133-270): it
takes world-space object and light meshes, materials in the 64-byte
``Material`` layout (src/core/Material.h:32-53), an optional environment image
and the camera, and builds the sampling tables and device buffers through the
C ABI.  ``PathIntegrator``, ``LightIntegrator`` and ``TripleIntegrator`` mirror
``NaivePathIntegrator``, ``LightPathIntegrator`` and ``TriplePathIntegrator``
(src/core/Integrator.h:68-172): ``render_one_pass``, ``reset``, ``get_frame``
and ``result_scale``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import call

LAMBERTIAN, PRINCIPLED, METAL_WORKFLOW, DIELECTRIC, THIN_DIELECTRIC = 0, 1, 2, 3, 4
NO_TEXTURE = -1


def material(type_: int = LAMBERTIAN, base_color=(1.0, 1.0, 1.0), roughness: float = 1.0, subsurface: float = 0.0,
             metallic: float = 0.0, specular: float = 1.0, specular_tint: float = 1.0, sheen: float = 0.0,
             sheen_tint: float = 1.0, clearcoat: float = 0.0, clearcoat_gloss: float = 0.0,
             ior: float = 1.5) -> np.ndarray:
    """One material record: 16 float32 in the layout of struct Material, with
    the defaults of src/core/Material.h:32-53 (type stored as int32 bits)."""
    rec = np.zeros(16, np.float32)
    rec[0:3] = base_color
    rec[3] = roughness
    rec[4:8] = (subsurface, metallic, specular, specular_tint)
    rec[8:12] = (sheen, sheen_tint, clearcoat, clearcoat_gloss)
    rec[12] = ior
    rec[13:14] = np.array([type_], np.int32).view(np.float32)
    return rec


def mat_tex(mat_index: int, tex_index: int = NO_TEXTURE) -> int:
    """(texIndex << 16) | matIndex as stored per triangle (Scene.cpp:168)."""
    return int(np.array([(tex_index << 16) | mat_index], np.int64).astype(np.int32)[0])


def alias_table(pdf) -> tuple[np.ndarray, np.ndarray]:
    """AliasTable::build<int32_t>(pdf) (src/math/AliasTable.h:12-54)."""
    pdf = np.ascontiguousarray(pdf, np.float32)
    alias = np.zeros(pdf.size, np.int32)
    prob = np.zeros(pdf.size, np.float32)
    call("zgl_alias_table_build", pdf.ctypes.data, pdf.size, alias.ctypes.data, prob.ctypes.data)
    return alias, prob


class SceneDesc(C.Structure):
    _fields_ = [
        ("obj_vertices", C.c_void_p), ("obj_n_vertices", C.c_size_t), ("obj_normals", C.c_void_p),
        ("obj_indices", C.c_void_p), ("obj_n_triangles", C.c_size_t), ("obj_mat_tex", C.c_void_p),
        ("materials", C.c_void_p), ("n_materials", C.c_size_t),
        ("light_vertices", C.c_void_p), ("light_n_vertices", C.c_size_t), ("light_normals", C.c_void_p),
        ("light_indices", C.c_void_p), ("light_n_triangles", C.c_size_t), ("light_first", C.c_void_p),
        ("light_power", C.c_void_p), ("n_light_instances", C.c_size_t),
        ("env_rgb", C.c_void_p), ("env_width", C.c_int32), ("env_height", C.c_int32), ("env_rotation", C.c_float),
        ("cam_pos", C.c_float * 3), ("cam_angle", C.c_float * 3), ("cam_fov", C.c_float),
        ("cam_lens_radius", C.c_float), ("cam_focal_dist", C.c_float),
        ("film_width", C.c_int32), ("film_height", C.c_int32), ("sampler", C.c_int32),
        ("obj_texcoords", C.c_void_p), ("n_textures", C.c_int32), ("tex_size", C.c_void_p), ("tex_rgb", C.c_void_p),
    ]


class IntegratorParams(C.Structure):
    _fields_ = [
        ("max_depth", C.c_int32), ("russian_roulette", C.c_int32), ("rr_start_depth", C.c_int32),
        ("sample_light", C.c_int32), ("light_env_uniform_sample", C.c_int32), ("light_portion", C.c_float),
        ("finite_sample", C.c_int32), ("max_sample", C.c_int32), ("blocks_per_pass", C.c_int32),
        ("loops_per_pass", C.c_int32),
    ]


def _f32(a, cols=3):
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, cols))


@dataclass
class SceneData:
    """World-space scene arrays (objects first, then lights), as flattened by
    Scene::createGLContext."""

    obj_vertices: np.ndarray
    obj_normals: np.ndarray
    obj_indices: np.ndarray
    obj_mat_tex: np.ndarray
    materials: np.ndarray            # (n, 16) float32
    light_vertices: np.ndarray
    light_normals: np.ndarray
    light_indices: np.ndarray
    light_first: np.ndarray          # uint32 offsets, n_instances + 1
    light_power: np.ndarray          # (n_instances, 3)
    film: tuple[int, int] = (256, 256)
    cam_pos: tuple = (0.0, 0.0, 0.0)
    cam_angle: tuple = (0.0, 0.0, 0.0)
    cam_fov: float = 45.0
    cam_lens_radius: float = 0.0
    cam_focal_dist: float = 1.0
    sampler: int = 1
    env_rgb: np.ndarray | None = None  # (H, W, 3) float32
    env_rotation: float = 0.0
    # albedo textures: per object vertex texcoords (n, 2) and 8-bit sRGB RGB
    # images (h, w, 3) uint8, top row first; a triangle uses texture
    # obj_mat_tex >> 16 (-1 = none)
    obj_texcoords: np.ndarray | None = None
    textures: list | None = None
    _keep: list = field(default_factory=list, repr=False)

    def normalized(self) -> "SceneData":
        self.obj_vertices = _f32(self.obj_vertices)
        self.obj_normals = _f32(self.obj_normals)
        self.obj_indices = np.ascontiguousarray(np.asarray(self.obj_indices, np.uint32).reshape(-1))
        self.obj_mat_tex = np.ascontiguousarray(np.asarray(self.obj_mat_tex, np.int32).reshape(-1))
        self.materials = _f32(self.materials, 16)
        self.light_vertices = _f32(self.light_vertices)
        self.light_normals = _f32(self.light_normals)
        self.light_indices = np.ascontiguousarray(np.asarray(self.light_indices, np.uint32).reshape(-1))
        self.light_first = np.ascontiguousarray(np.asarray(self.light_first, np.uint32).reshape(-1))
        self.light_power = _f32(self.light_power)
        if self.env_rgb is not None:
            self.env_rgb = np.ascontiguousarray(np.asarray(self.env_rgb, np.float32))
        if self.obj_texcoords is not None:
            self.obj_texcoords = _f32(self.obj_texcoords, 2)
        if self.textures:
            self.textures = [np.ascontiguousarray(np.asarray(t, np.uint8).reshape(t.shape[0], t.shape[1], 3))
                             for t in self.textures]
        return self

    def desc(self) -> SceneDesc:
        self.normalized()
        d = SceneDesc()
        p = lambda a: a.ctypes.data if a is not None and a.size else None  # noqa: E731
        d.obj_vertices, d.obj_n_vertices = p(self.obj_vertices), self.obj_vertices.shape[0]
        d.obj_normals = p(self.obj_normals)
        d.obj_indices, d.obj_n_triangles = p(self.obj_indices), self.obj_indices.size // 3
        d.obj_mat_tex = p(self.obj_mat_tex)
        d.materials, d.n_materials = p(self.materials), self.materials.shape[0]
        d.light_vertices, d.light_n_vertices = p(self.light_vertices), self.light_vertices.shape[0]
        d.light_normals = p(self.light_normals)
        d.light_indices, d.light_n_triangles = p(self.light_indices), self.light_indices.size // 3
        d.light_first = p(self.light_first)
        d.light_power, d.n_light_instances = p(self.light_power), self.light_power.shape[0]
        if self.env_rgb is not None:
            d.env_rgb = self.env_rgb.ctypes.data
            d.env_height, d.env_width = self.env_rgb.shape[0], self.env_rgb.shape[1]
        d.env_rotation = self.env_rotation
        d.cam_pos = (C.c_float * 3)(*self.cam_pos)
        d.cam_angle = (C.c_float * 3)(*self.cam_angle)
        d.cam_fov, d.cam_lens_radius, d.cam_focal_dist = self.cam_fov, self.cam_lens_radius, self.cam_focal_dist
        d.film_width, d.film_height = self.film
        d.sampler = self.sampler
        d.obj_texcoords = p(self.obj_texcoords)
        if self.textures:
            size = np.array([(t.shape[1], t.shape[0]) for t in self.textures], np.int32).reshape(-1)
            rgb = np.concatenate([t.reshape(-1) for t in self.textures])
            self._keep[:] = [size, rgb]
            d.n_textures, d.tex_size, d.tex_rgb = len(self.textures), size.ctypes.data, rgb.ctypes.data
        return d

    # flattened arrays (objects then lights), for checkers
    def flat(self):
        self.normalized()
        nvo = self.obj_vertices.shape[0]
        v = np.concatenate([self.obj_vertices, self.light_vertices]).astype(np.float32)
        n = np.concatenate([self.obj_normals, self.light_normals]).astype(np.float32)
        idx = np.concatenate([self.obj_indices, self.light_indices + np.uint32(nvo)]).astype(np.uint32)
        return v, n, idx


class Scene:
    """Device-resident scene (owner of a ``zgl_scene`` handle)."""

    TABLES = {
        "info": np.int64, "vertices": np.float32, "normals": np.float32, "indices": np.uint32,
        "mat_tex": np.int32, "materials": np.float32,
        "light_power": np.float32, "light_alias": np.int32, "light_prob": np.float32, "env_alias": np.int32,
        "env_prob": np.float32, "env_texels": np.float32, "sobol": np.uint32, "noise": np.float32,
        "pixel_seeds": np.uint32, "camera": np.float32, "scalars": np.float32, "tex_scale": np.float32,
        "srgb_lut": np.float32, "texcoords": np.float32, "tex_texels": np.uint32,
    }

    def __init__(self, data: SceneData, host_only: bool = False):
        self.data = data
        desc = data.desc()
        h = C.c_void_p()
        call("zgl_scene_create", C.byref(desc), 1 if host_only else 0, C.byref(h))
        self._h = h
        self._info()

    @classmethod
    def load(cls, path, host_only: bool = False) -> "Scene":
        """Scene::load of a scene XML file (OBJ models, PFM environment)."""
        self = cls.__new__(cls)
        self.data = None
        h = C.c_void_p()
        call("zgl_scene_load_xml", str(path).encode(), 1 if host_only else 0, C.byref(h))
        self._h = h
        self._info()
        return self

    def _info(self):
        info = np.empty(13, np.int64)
        call("zgl_scene_export", self._h, b"info", info.ctypes.data, info.nbytes)
        self.info = {k: int(v) for k, v in zip(
            ["film_w", "film_h", "vertices", "obj_vertices", "triangles", "obj_triangles", "light_triangles",
             "materials", "env_w", "env_h", "textures", "tex_w", "tex_h"], info)}
        self.film = (self.info["film_w"], self.info["film_h"])

    def table_size(self, name: str) -> int:
        i = self.info
        nl, (W, H), ew, eh = i["light_triangles"], self.film, i["env_w"], i["env_h"]
        return {
            "info": 13, "vertices": 3 * i["vertices"], "normals": 3 * i["vertices"], "indices": 3 * i["triangles"],
            "mat_tex": i["obj_triangles"], "materials": 16 * i["materials"],
            "light_power": nl * 3, "light_alias": nl, "light_prob": nl,
            "env_alias": (ew + 1) * eh, "env_prob": (ew + 1) * eh, "env_texels": ew * eh * 3,
            "sobol": 256 * 32, "noise": W * H * 2, "pixel_seeds": W * H * 2, "camera": 19, "scalars": 4,
            "tex_scale": 2 * i["textures"], "srgb_lut": 256, "texcoords": 2 * i["obj_vertices"],
            "tex_texels": i["textures"] * i["tex_w"] * i["tex_h"],
        }[name]

    def export(self, name: str) -> np.ndarray:
        out = np.empty(self.table_size(name), self.TABLES[name])
        call("zgl_scene_export", self._h, name.encode(), out.ctypes.data if out.size else C.c_void_p(1),
             out.nbytes)
        return out

    def close(self):
        if self._h:
            call("zgl_scene_destroy", self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h


def default_params(**kw) -> IntegratorParams:
    p = IntegratorParams()
    call("zgl_integrator_params_default", C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class IntegratorState(C.Structure):
    """zgl_integrator_state: the counters of a checkpoint."""

    _fields_ = [("kind", C.c_int32), ("cur_sample", C.c_int32), ("free_counter", C.c_int32),
                ("finished", C.c_int32), ("sample_per_pixel", C.c_float)]


class PathIntegrator:
    """NaivePathIntegrator (src/core/Integrator.h:68-91) on the GPU."""

    KIND = 0

    def __init__(self, scene: Scene, params: IntegratorParams | None = None, **kw):
        self.scene = scene
        self.params = params or default_params(**kw)
        h = C.c_void_p()
        call("zgl_integrator_create", scene.handle, self.KIND, C.byref(self.params), C.byref(h))
        self._h = h

    def render_one_pass(self, stream=None) -> None:
        from .accel import _stream_handle

        call("zgl_integrator_render_pass", self._h, _stream_handle(stream))

    def render_passes(self, passes: int, stream=None) -> None:
        """`passes` consecutive passes (one launch for the path tracer)."""
        from .accel import _stream_handle

        call("zgl_integrator_render_passes", self._h, int(passes), _stream_handle(stream))

    def reset(self) -> None:
        call("zgl_integrator_reset", self._h)

    def get_frame(self, out=None, stream=None):
        """(RGBA sum image (H, W, 4), samples)."""
        from .accel import _ptr, _stream_handle

        W, H = self.scene.film
        if out is None:
            out = np.empty((H, W, 4), np.float32)
        spp = C.c_int32()
        call("zgl_integrator_frame", self._h, _ptr(out), C.byref(spp), _stream_handle(stream))
        return out, spp.value

    def result_scale(self) -> float:
        v = C.c_float()
        call("zgl_integrator_result_scale", self._h, C.byref(v))
        return v.value

    def save(self, stream=None):
        """Checkpoint: (counters dict, running sum as a float32 array)."""
        from .accel import _stream_handle

        n = C.c_size_t()
        call("zgl_integrator_state_size", self._h, C.byref(n))
        total = np.empty(n.value, np.float32)
        st = IntegratorState()
        call("zgl_integrator_save", self._h, C.byref(st), total.ctypes.data, _stream_handle(stream))
        return {k: getattr(st, k) for k, _ in st._fields_}, total

    def restore(self, state: dict, total, stream=None) -> None:
        """Continue from a checkpoint taken by :meth:`save`."""
        from .accel import _ptr, _stream_handle

        n = C.c_size_t()
        call("zgl_integrator_state_size", self._h, C.byref(n))
        if total.size != n.value:
            raise ValueError(f"checkpoint holds {total.size} floats, this integrator needs {n.value}")
        st = IntegratorState(**state)
        call("zgl_integrator_restore", self._h, C.byref(st), _ptr(total), _stream_handle(stream))

    def close(self):
        if self._h:
            call("zgl_integrator_destroy", self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LightIntegrator(PathIntegrator):
    """LightPathIntegrator (src/core/Integrator.h:103-129): the particle
    tracer; the frame is the film sum, result_scale() = 1 / samplePerPixel."""

    KIND = 1


class TripleIntegrator(PathIntegrator):
    """TriplePathIntegrator (src/core/Integrator.h:145-172): MIS-weighted
    (s=0) + (s=1) + (t=1) strategies, camera pass then light pass."""

    KIND = 2


class RenderRequest(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("spp", C.c_int32), ("params", IntegratorParams), ("frame", C.c_void_p)]


class BatchConfig(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("queue_capacity", C.c_int32), ("regen_threshold", C.c_int32),
                ("schedule", C.c_int32), ("scratch_mib", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _gpu_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        pass
    return "cuda"


def autotune_cache_key(gpu: str, summary) -> str:
    """Cache key of a batch: GPU name and the workload class, i.e. request
    count, total samples and largest scene (triangles), each rounded to a
    power of two.  ``summary`` lists (triangles, pixels, spp) per request."""
    import math

    def p2(x):
        return 0 if x <= 1 else int(round(math.log2(x)))

    n = len(summary)
    samples = sum(px * spp for _, px, spp in summary)
    tris = max((t for t, _, _ in summary), default=0)
    return f"{gpu}|requests 2^{p2(n)}|samples 2^{p2(samples)}|triangles 2^{p2(tris)}"


def cached_autotune(path, key: str, tune, apply) -> dict:
    """The configuration stored under ``key`` in the JSON file ``path``
    (applied with ``apply``), or ``tune()``'s result, which is then stored.
    The file is rewritten atomically; an unreadable file counts as empty."""
    import json
    import os

    table = {}
    try:
        with open(path) as f:
            table = json.load(f)
        if not isinstance(table, dict):
            table = {}
    except (OSError, ValueError):
        table = {}
    if key in table:
        cfg = {k: int(v) for k, v in table[key].items()}
        apply(cfg)
        return cfg
    cfg = tune()
    table[key] = cfg
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return cfg


class BatchRenderer:
    """Many path-tracing requests in persistent launches (zgl_batch_*).

    ``requests`` is a list of ``(scene, spp, params, frame)`` with ``frame`` a
    CUDA float32 tensor of shape (H, W, 4); after :meth:`render` each frame
    holds what :class:`PathIntegrator` holds after ``spp`` passes."""

    def __init__(self, requests, **config):
        from .accel import _ptr

        arr = (RenderRequest * len(requests))()
        self._keep = []
        self._summary = [(int(scene.info["triangles"]), int(scene.film[0]) * int(scene.film[1]), int(spp))
                         for scene, spp, _, _ in requests]
        for i, (scene, spp, params, frame) in enumerate(requests):
            arr[i].scene = scene.handle.value
            arr[i].spp = spp
            arr[i].params = params if isinstance(params, IntegratorParams) else default_params(**params)
            arr[i].frame = _ptr(frame)
            self._keep.append((scene, frame))
        cfg = BatchConfig()
        call("zgl_batch_config_default", C.byref(cfg))
        for k, v in config.items():
            setattr(cfg, k, v)
        h = C.c_void_p()
        call("zgl_batch_create", arr, len(requests), C.byref(cfg), C.byref(h))
        self._h = h

    def render(self, stream=None) -> None:
        from .accel import _stream_handle

        call("zgl_batch_render", self._h, _stream_handle(stream))

    def autotune(self, stream=None, cache=None) -> dict:
        """Pick the fastest configuration (zgl_batch_autotune) and keep it.

        With ``cache`` (a JSON file path) the choice is stored under a key of
        the GPU's name and the workload class (request count, total samples
        and largest scene, each rounded to a power of two); a later call with
        the same key reuses it without timing anything."""
        from .accel import _stream_handle

        def tune():
            cfg = BatchConfig()
            call("zgl_batch_autotune", self._h, _stream_handle(stream), C.byref(cfg))
            return cfg.as_dict()

        if cache is None:
            return tune()
        key = autotune_cache_key(_gpu_name(), self._summary)
        return cached_autotune(cache, key, tune, lambda c: self.set_config(**c))

    def config(self) -> dict:
        cfg = BatchConfig()
        call("zgl_batch_get_config", self._h, C.byref(cfg))
        return cfg.as_dict()

    def set_config(self, **config) -> None:
        cfg = BatchConfig()
        call("zgl_batch_get_config", self._h, C.byref(cfg))
        for k, v in config.items():
            setattr(cfg, k, v)
        call("zgl_batch_set_config", self._h, C.byref(cfg))

    def close(self):
        if self._h:
            call("zgl_batch_destroy", self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DiffRenderer:
    """Differentiable path tracer over a :class:`Scene` (zgl_diff_*).

    :meth:`forward` renders the mean of the path tracer's first ``spp``
    samples into a CUDA float32 tensor (H, W, 3); :meth:`backward` takes the
    image adjoint (H, W, 3) and returns the gradient of
    ``sum(adjoint * image)`` with respect to :meth:`params` by path replay.
    Parameter layout: per material (baseColor r, g, b, raw roughness,
    metallic, specular), then per light instance (power r, g, b)."""

    MAT_PARAMS = 6

    def __init__(self, scene: Scene, spp: int, params: IntegratorParams | None = None, **kw):
        self.scene = scene
        self.spp = spp
        self.params_struct = params or default_params(**kw)
        h = C.c_void_p()
        call("zgl_diff_create", scene.handle, C.byref(self.params_struct), spp, C.byref(h))
        self._h = h
        n = C.c_int32()
        call("zgl_diff_param_count", self._h, C.byref(n))
        self.n_params = n.value

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        call("zgl_diff_get_params", self._h, out.ctypes.data)
        return out

    def set_params(self, values) -> None:
        from .accel import _ptr

        if getattr(values, "shape", None) != (self.n_params,):
            raise ValueError(f"expected {self.n_params} parameters")
        if not hasattr(values, "data_ptr"):
            values = np.ascontiguousarray(values, np.float32)
        elif str(values.dtype) != "torch.float32":
            raise ValueError("parameters must be float32")
        call("zgl_diff_set_params", self._h, _ptr(values))

    def forward(self, out=None, stream=None):
        import torch

        from .accel import _ptr, _stream_handle

        W, H = self.scene.film
        if out is None:
            out = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
        call("zgl_diff_forward", self._h, _ptr(out), _stream_handle(stream))
        return out

    def backward(self, d_image, out=None, stream=None):
        import torch

        from .accel import _ptr, _stream_handle

        d_image = d_image.contiguous()
        if out is None:
            out = torch.empty(self.n_params, dtype=torch.float32, device=d_image.device)
        call("zgl_diff_backward", self._h, _ptr(d_image), _ptr(out), _stream_handle(stream))
        return out

    def step_l2(self, target, loss_scale=None, image=None, grad=None, loss=None, stream=None):
        """Fused forward + adjoint of loss = loss_scale * sum((image - target)^2)
        (zgl_diff_step_l2; loss_scale defaults to 1 / target.numel(), the
        mean squared error).  Returns (image, grad, loss) as CUDA tensors."""
        import torch

        from .accel import _ptr, _stream_handle

        target = target.contiguous()
        W, H = self.scene.film
        if loss_scale is None:
            loss_scale = 1.0 / target.numel()
        if image is None:
            image = torch.empty((H, W, 3), dtype=torch.float32, device=target.device)
        if grad is None:
            grad = torch.empty(self.n_params, dtype=torch.float32, device=target.device)
        if loss is None:
            loss = torch.empty(1, dtype=torch.float32, device=target.device)
        call("zgl_diff_step_l2", self._h, _ptr(target), float(loss_scale), _ptr(image), _ptr(grad), _ptr(loss),
             _stream_handle(stream))
        return image, grad, loss

    def close(self):
        if self._h:
            call("zgl_diff_destroy", self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
