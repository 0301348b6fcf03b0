"""ctypes binding of libfvc.so (include/fvc.h).

The library is the product: if it is missing or fails to load this module
raises; there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

c_float, c_int, c_u8 = C.c_float, C.c_int, C.c_uint8


class Float2(C.Structure):
    _pack_ = 8
    _fields_ = [("x", c_float), ("y", c_float)]


class Float3(C.Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float)]


class Float4(C.Structure):
    _fields_ = [("x", c_float), ("y", c_float), ("z", c_float), ("w", c_float)]


class Int2(C.Structure):
    _fields_ = [("x", c_int), ("y", c_int)]


class Int3(C.Structure):
    _fields_ = [("x", c_int), ("y", c_int), ("z", c_int)]


class CameraMatrix(C.Structure):
    _fields_ = [("m0", Float4), ("m1", Float4), ("m2", Float4)]


class SceneInfo(C.Structure):
    _fields_ = [("grid_resolution", c_int), ("grid_nlvl", c_int), ("vals_per_lvl", c_int), ("normalized", c_u8),
                ("aabb_from", Float3), ("aabb_to", Float3), ("contraction_aabb_from", Float3),
                ("contraction_aabb_to", Float3), ("contraction_type", c_int), ("is_open_gl", c_u8),
                ("alpha_thre", c_float)]


class StepsizeInfo(C.Structure):
    _fields_ = [(n, c_float) for n in ["cone_angle", "log1p_c", "stepsize", "near", "near_i", "far", "dt_min", "dt_max",
                                       "t_min", "t_max", "i_min", "i_max"]]


class CameraInfo(C.Structure):
    _fields_ = [("resolution", Int2), ("is_open_gl", c_u8), ("_pad0", c_u8 * 7), ("focal", Float2),
                ("principal", Float2), ("_pad1", c_u8 * 0), ("cam2world", CameraMatrix),
                ("world2cam", CameraMatrix), ("aperature", c_float), ("focus_z", c_float), ("_pad2", c_u8 * 8)]


class RaymarchInfo(C.Structure):
    _fields_ = [("cam_info", CameraInfo), ("next_cam_info", CameraInfo), ("stepsize_info", StepsizeInfo),
                ("sample_index", c_int), ("motion_blur", c_u8), ("deterministic", c_u8), ("_pad", c_u8 * 10)]


class RayResult(C.Structure):
    _fields_ = [("r", c_float), ("g", c_float), ("b", c_float), ("transmittance", c_float)]


class CacheSettings(C.Structure):
    _fields_ = [("interpol_variant", c_int), ("interpol_function", c_int), ("use_hw_interpol", c_u8),
                ("reweight_intermediates", c_u8), ("disable_reweighting_first_intermediate", c_u8),
                ("use_inter_brick_interpolation", c_u8)]


class RenderOutputs(C.Structure):
    _fields_ = [("image_rgba8", C.c_void_p), ("results", C.c_void_p), ("ray_counts", C.c_void_p),
                ("contrib_resample", C.c_void_p), ("contrib_cache", C.c_void_p)]


class RenderStats(C.Structure):
    _fields_ = [("samples_ppx", C.c_double), ("n_samples", C.c_longlong), ("n_resamples", C.c_longlong),
                ("n_cache_hits", C.c_longlong), ("n_dropped", C.c_longlong), ("n_steps", C.c_longlong),
                ("n_rounds", c_int), ("guard_flags", c_int), ("n_launches", C.c_longlong),
                ("n_timed_launches", c_int), ("timed_kernel_ms", C.c_float),
                ("n_miss_outside_fov", C.c_longlong), ("n_miss_outside_depth", C.c_longlong),
                ("n_miss_before_near", C.c_longlong), ("n_miss_beyond_known", C.c_longlong),
                ("n_drop_brick_unset", C.c_longlong), ("n_drop_voxel_empty", C.c_longlong),
                ("n_drop_alpha", C.c_longlong), ("n_timed_adjoint_launches", c_int), ("timed_adjoint_ms", C.c_float)]


class ModelProps(C.Structure):
    _fields_ = [("first_latent_is_density", c_int), ("head_hidden_layers", c_int), ("n_levels", c_int),
                ("n_latents", c_int), ("occupancy_bitfield", C.c_void_p), ("occupancy_bytes", C.c_size_t)]


class AutotuneResult(C.Structure):
    _fields_ = [("m_tile", c_int), ("steps_per_iter", c_int), ("rows_per_iteration", C.c_longlong), ("ms", C.c_float),
                ("n_candidates", c_int), ("batch_rows", c_int), ("reserved", c_int)]


class CacheStats(C.Structure):
    _fields_ = [("n_bricks_set", c_int), ("n_bricks_reserved", c_int), ("n_bricks_demanded", c_int),
                ("overflow", c_int), ("n_iterations", c_int), ("n_launches", c_int), ("n_samples", C.c_longlong)]


assert C.sizeof(SceneInfo) == 76 and C.sizeof(StepsizeInfo) == 48
assert C.sizeof(CameraInfo) == 144 and CameraInfo.cam2world.offset == 32 and CameraInfo.world2cam.offset == 80
assert C.sizeof(RenderStats) == 136 and C.sizeof(CacheStats) == 32 and C.sizeof(AutotuneResult) == 32
assert C.sizeof(RaymarchInfo) == 352 and RaymarchInfo.stepsize_info.offset == 288 and RaymarchInfo.sample_index.offset == 336

FVC_OK = 0
ERRORS = {1: "CUDA", 2: "CONFIG", 3: "OOM", 4: "CACHE_UNINIT", 5: "TIMEOUT", 6: "ARG", 7: "IO", 8: "GUARD"}

# exported symbol -> (restype, argtypes)
P = C.c_void_p
PP = C.POINTER(C.c_void_p)
SIGNATURES = {
    "fvc_last_error": (C.c_char_p, []),
    "fvc_version": (C.c_char_p, []),
    "fvc_model_load": (c_int, [C.c_char_p, PP]),
    "fvc_ingp_export": (c_int, [C.c_char_p, C.c_char_p]),
    "fvc_model_destroy": (None, [P]),
    "fvc_model_info": (c_int, [P, C.POINTER(SceneInfo), C.POINTER(StepsizeInfo)]),
    "fvc_debug_fail_allocation": (c_int, [C.c_longlong]),
    "fvc_selftest_wait_timeout": (c_int, [C.c_double, C.POINTER(C.c_double)]),
    "fvc_selftest_division": (c_int, [P, P, c_int, P, P]),
    "fvc_stepsize_setup": (c_int, [C.POINTER(SceneInfo), C.POINTER(StepsizeInfo)]),
    "fvc_model_density": (c_int, [P, P, c_int, P]),
    "fvc_model_inference": (c_int, [P, P, P, c_int, P]),
    "fvc_model_debug_encode": (c_int, [P, P, c_int, P, P]),
    "fvc_renderer_create": (c_int, [P, c_int, PP]),
    "fvc_renderer_destroy": (None, [P]),
    "fvc_renderer_resize": (c_int, [P, c_int, c_int]),
    "fvc_renderer_set_stream": (c_int, [P, P]),
    "fvc_render_device": (c_int, [P, C.POINTER(RaymarchInfo), C.POINTER(RenderOutputs)]),
    "fvc_render": (c_int, [P, C.POINTER(RaymarchInfo), C.POINTER(RenderOutputs)]),
    "fvc_renderer_set_max_samples_per_ray": (c_int, [P, c_int]),
    "fvc_render_stats": (c_int, [P, C.POINTER(RenderStats)]),
    "fvc_cache_create": (c_int, [PP]),
    "fvc_cache_destroy": (None, [P]),
    "fvc_renderer_set_caches": (c_int, [P, P, P]),
    "fvc_cache_resize": (c_int, [P, c_int, c_int, C.POINTER(StepsizeInfo)]),
    "fvc_renderer_set_cache_settings": (c_int, [P, C.POINTER(CacheSettings)]),
    "fvc_cache_build": (c_int, [P, C.POINTER(RaymarchInfo)]),
    "fvc_cache_build_per_ray": (c_int, [P, C.POINTER(RaymarchInfo)]),
    "fvc_cache_swap": (c_int, [P]),
    "fvc_cache_stats": (c_int, [P, C.POINTER(CacheStats)]),
    "fvc_renderer_set_render_mode": (c_int, [P, c_int]),
    "fvc_cache_read": (c_int, [P, P, C.POINTER(C.c_size_t), P, C.POINTER(C.c_size_t), P, C.POINTER(C.c_size_t)]),
    "fvc_cache_dims": (c_int, [P, C.POINTER(Int3), C.POINTER(Int3), C.POINTER(Int3)]),
    "fvc_render_noalloc": (c_int, [P, C.POINTER(RaymarchInfo), C.POINTER(RenderOutputs), P]),
    "fvc_renderer_set_network_path": (c_int, [P, c_int]),
    "fvc_renderer_set_build_network_path": (c_int, [P, c_int]),
    "fvc_renderer_set_tiling": (c_int, [P, c_int, c_int]),
    "fvc_renderer_set_fused_classify": (c_int, [P, c_int]),
    "fvc_renderer_set_empty_space_skipping": (c_int, [P, c_int]),
    "fvc_cache_set_sizing": (c_int, [P, c_int, C.c_float]),
    "fvc_renderer_set_kernel_timing": (c_int, [P, c_int]),
    "fvc_renderer_set_precision": (c_int, [P, c_int]),
    "fvc_render_batch": (c_int, [P, C.POINTER(RaymarchInfo), c_int, C.POINTER(RenderOutputs)]),
    "fvc_render_batch_cached": (c_int, [P, C.POINTER(RaymarchInfo), c_int, PP, C.POINTER(RenderOutputs)]),
    "fvc_renderer_autotune": (c_int, [P, C.POINTER(RaymarchInfo), c_int, C.POINTER(RenderOutputs), C.POINTER(AutotuneResult)]),
    "fvc_renderer_set_autotune_space": (c_int, [P, C.POINTER(c_int), c_int, C.POINTER(c_int), c_int, C.POINTER(c_int), c_int]),
    "fvc_model_properties": (c_int, [P, C.POINTER(ModelProps)]),
    "fvc_renderer_synchronize": (c_int, [P]),
    "fvc_grad_create": (c_int, [P, PP]),
    "fvc_grad_destroy": (None, [P]),
    "fvc_grad_zero": (c_int, [P]),
    "fvc_grad_sizes": (c_int, [P, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "fvc_grad_read": (c_int, [P, P, P, P]),
    "fvc_grad_cache_latents": (c_int, [P, P, C.POINTER(C.c_size_t)]),
    "fvc_render_backward": (c_int, [P, P, C.POINTER(RaymarchInfo), P, c_int, P, C.POINTER(C.c_double), P]),
}

_lib = None


class FvcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fvc error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


def lib_path() -> str:
    return os.environ.get("FVC_LIB", _build.LIB)


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libfvc.so (building it first when absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path) and build_if_missing:
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libfvc.so not found at {path}: build it with `python -m frustumvolumecaching_gb300.build`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != FVC_OK:
        raise FvcError(rc, load().fvc_last_error().decode())


def ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return int(a)
