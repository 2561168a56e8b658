"""ctypes binding of libzgl.so (the C ABI declared in include/zgl.h).

The library is the only compute path: there is no Python or CPU fallback.  If
``zillumgl_gb300/_build/libzgl.so`` is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libzgl.so"

ZGL_OK = 0
STATUS_NAMES = {
    0: "OK",
    1: "INVALID_ARG",
    2: "CUDA",
    3: "OOM",
    4: "TIMEOUT",
    5: "PARSE",
    6: "STATE",
}

_lock = threading.Lock()
_lib: C.CDLL | None = None

c_float_p = C.POINTER(C.c_float)
c_int32_p = C.POINTER(C.c_int32)
c_uint32_p = C.POINTER(C.c_uint32)
c_uint8_p = C.POINTER(C.c_uint8)
c_size_t_p = C.POINTER(C.c_size_t)


class ZglError(RuntimeError):
    """A libzgl call returned a status other than ZGL_OK."""

    def __init__(self, status: int, message: str):
        super().__init__(f"zgl status {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# name -> (restype, argtypes); kept in the order of include/zgl.h
SIGNATURES: dict[str, tuple] = {
    "zgl_version": (C.c_int32, []),
    "zgl_last_error": (C.c_char_p, []),
    "zgl_accel_build": (C.c_int32, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]),
    "zgl_accel_build_device": (C.c_int32, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int32, C.c_void_p,
                                           C.POINTER(C.c_void_p)]),
    "zgl_accel_node_count": (C.c_int32, [C.c_void_p, c_size_t_p]),
    "zgl_accel_export": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_accel_destroy": (C.c_int32, [C.c_void_p]),
    "zgl_bvh_build_host": (C.c_int32, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "zgl_accel_set_trace_schedule": (C.c_int32, [C.c_void_p, C.c_int32]),
    "zgl_trace_closest": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "zgl_trace_any": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                  C.c_void_p]),
    "zgl_trace_count": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_trace_closest_noalloc": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                              C.c_void_p, C.c_void_p]),
    "zgl_scene_create": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "zgl_scene_export": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_size_t]),
    "zgl_scene_load_xml": (C.c_int32, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "zgl_scene_destroy": (C.c_int32, [C.c_void_p]),
    "zgl_alias_table_build": (C.c_int32, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "zgl_integrator_params_default": (C.c_int32, [C.c_void_p]),
    "zgl_integrator_create": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "zgl_integrator_render_pass": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_integrator_render_passes": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p]),
    "zgl_integrator_reset": (C.c_int32, [C.c_void_p]),
    "zgl_integrator_frame": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_integrator_result_scale": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_integrator_destroy": (C.c_int32, [C.c_void_p]),
    "zgl_integrator_state_size": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_integrator_save": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_integrator_restore": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_batch_config_default": (C.c_int32, [C.c_void_p]),
    "zgl_batch_create": (C.c_int32, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "zgl_batch_render": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_batch_autotune": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_batch_set_config": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_batch_get_config": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_batch_destroy": (C.c_int32, [C.c_void_p]),
    "zgl_diff_create": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "zgl_diff_param_count": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int32)]),
    "zgl_diff_get_params": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_diff_set_params": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "zgl_diff_forward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_diff_backward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "zgl_diff_step_l2": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    "zgl_diff_destroy": (C.c_int32, [C.c_void_p]),
    "zgl_postprocess": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_int32, C.c_void_p,
                                    C.c_void_p]),
    "zgl_measure_l2_read": (C.c_int32, [C.c_size_t, C.c_int32, C.POINTER(C.c_double), C.c_void_p]),
}


def lib() -> C.CDLL:
    """Loads libzgl.so once (raising if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise ZglError(6, f"{LIB_PATH} is missing: run __graft_entry__.build() to compile the CUDA "
                                  "library (there is no fallback path)")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def check(status: int) -> None:
    if status != ZGL_OK:
        msg = lib().zgl_last_error().decode(errors="replace")
        raise ZglError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
