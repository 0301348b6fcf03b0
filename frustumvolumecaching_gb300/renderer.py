"""Python mirror of the reference's renderer API over the C ABI.

Same names and argument meanings as the reference's C++ classes
(include/renderer.h, performance_renderer.h, cache_renderer.h,
cache_performance_renderer.h, include/loader.h), so parity tests read like
the reference's own call sites (src/eval.cu:208-227, 285-478):

    loader = load_data(model_dir)
    renderer = PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    renderer.resizeRenderbuffers((W, H))
    renderer.render(rm_info, image_buffer)

Errors are raised as FvcError (the reference throws std::runtime_error).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .camera import camera_dict, inverse

RENDERER_BASIC, RENDERER_PERFORMANCE, RENDERER_CACHE_PERFORMANCE, RENDERER_CACHE_BASIC = 0, 1, 2, 3


class NerfNetwork:
    """Loaded model (NerfNetwork<half> + the occupancy grid it came with)."""

    def __init__(self, path: str):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.fvc_model_load(path.encode(), C.byref(h)))
        self.handle = h
        self.path = path
        self.scene_info = L.SceneInfo()
        self.stepsize_info = L.StepsizeInfo()
        L.check(lib.fvc_model_info(h, C.byref(self.scene_info), C.byref(self.stepsize_info)))

    def inference(self, pos: np.ndarray, dir01: np.ndarray) -> np.ndarray:
        """NerfNetwork::inference at given inputs: [n,4] = rgb logits, log-density."""
        pos = np.ascontiguousarray(pos, np.float32)
        dir01 = np.ascontiguousarray(dir01, np.float32)
        out = np.zeros((pos.shape[0], 4), np.float32)
        L.check(L.load().fvc_model_inference(self.handle, L.ptr(pos), L.ptr(dir01), pos.shape[0], L.ptr(out)))
        return out

    def density(self, pos: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float32)
        out = np.zeros(pos.shape[0], np.float32)
        L.check(L.load().fvc_model_density(self.handle, L.ptr(pos), pos.shape[0], L.ptr(out)))
        return out

    def properties(self) -> dict:
        """First-latent-is-density, head depth, hash levels, latents and the
        device occupancy bitfield (fvc_model_properties)."""
        p = L.ModelProps()
        L.check(L.load().fvc_model_properties(self.handle, C.byref(p)))
        return {k: getattr(p, k) for k, _ in p._fields_}

    def debug_encode(self, pos: np.ndarray):
        pos = np.ascontiguousarray(pos, np.float32)
        f = np.zeros((pos.shape[0], 32), np.float32)
        b = np.zeros((pos.shape[0], 16), np.float32)
        L.check(L.load().fvc_model_debug_encode(self.handle, L.ptr(pos), pos.shape[0], L.ptr(f), L.ptr(b)))
        return f, b

    def __del__(self):
        if getattr(self, "handle", None) and L._lib is not None:
            L._lib.fvc_model_destroy(self.handle)
            self.handle = None


@dataclass
class LoaderData:
    """LoaderData, include/loader.h:32-47."""
    scene_info: L.SceneInfo
    stepsize_info: L.StepsizeInfo
    nerf_network: NerfNetwork
    data_source: str = "nerfacc"  # DataSource INGP / NERFACC (include/loader.h:15-19)

    @property
    def occupancy_grid_morton_bitfield(self):
        return self.nerf_network


def load_data(path: str) -> LoaderData:
    """load_data(fs::path, LoaderData&), src/loader.cu:287-300: an instant-ngp
    snapshot (``.ingp``) or a nerfacc export directory."""
    net = NerfNetwork(str(path))
    src = "ingp" if os.path.splitext(str(path))[1] == ".ingp" else "nerfacc"
    return LoaderData(net.scene_info, net.stepsize_info, net, src)


def ingp_export(snapshot: str, export_dir: str) -> str:
    """Rewrites an instant-ngp snapshot as the equivalent nerfacc export
    directory (host only; no GPU needed)."""
    L.check(L.load().fvc_ingp_export(str(snapshot).encode(), str(export_dir).encode()))
    return str(export_dir)


def camera_info(cam: dict) -> L.CameraInfo:
    """CameraInfo from a camera dict of frustumvolumecaching_gb300.camera."""
    ci = L.CameraInfo()
    ci.resolution.x, ci.resolution.y = cam["resolution"]
    ci.is_open_gl = int(bool(cam["is_open_gl"]))
    ci.focal.x, ci.focal.y = cam["focal"]
    ci.principal.x, ci.principal.y = cam["principal"]
    c2w = np.asarray(cam["cam2world"], np.float32)
    w2c = np.asarray(cam.get("world2cam", inverse(c2w)), np.float32)
    for r, name in enumerate(["m0", "m1", "m2"]):
        m = getattr(ci.cam2world, name)
        m.x, m.y, m.z, m.w = [float(v) for v in c2w[r]]
        m = getattr(ci.world2cam, name)
        m.x, m.y, m.z, m.w = [float(v) for v in w2c[r]]
    ci.aperature = float(cam.get("aperature", 0.0))
    ci.focus_z = float(cam.get("focus_z", 1.0))
    return ci


def raymarch_info(cam: dict, stepsize_info: L.StepsizeInfo, sample_index: int | None = None) -> L.RaymarchInfo:
    """RaymarchInfo as src/eval.cu:160-167 builds it: deterministic, no motion
    blur, unless the camera dict says otherwise (keys "deterministic",
    "motion_blur", "sample_index", "aperature", "focus_z", and
    "next_cam2world" for the motion-blur end pose)."""
    rm = L.RaymarchInfo()
    rm.cam_info = camera_info(cam)
    nxt = dict(cam)
    if "next_cam2world" in cam:
        nxt["cam2world"] = cam["next_cam2world"]
        nxt.pop("world2cam", None)
    rm.next_cam_info = camera_info(nxt)
    rm.stepsize_info = stepsize_info
    rm.sample_index = int(cam.get("sample_index", 0) if sample_index is None else sample_index)
    rm.motion_blur = int(bool(cam.get("motion_blur", False)))
    rm.deterministic = int(bool(cam.get("deterministic", True)))
    return rm


class RenderBuffer:
    """Headless image buffer (ImageBuffer, include/util/image_buffer.h) in host
    memory: uchar4 image, float rgb+transmittance per ray, per-ray counts."""

    def __init__(self, resolution):
        W, H = resolution
        self.resolution = (W, H)
        self.image = np.zeros((H, W, 4), np.uint8)
        self.results = np.zeros((H, W, 4), np.float32)
        self.ray_counts = np.zeros((H, W, 4), np.int32)

    def outputs(self) -> L.RenderOutputs:
        o = L.RenderOutputs()
        o.image_rgba8, o.results, o.ray_counts = L.ptr(self.image), L.ptr(self.results), L.ptr(self.ray_counts)
        return o


class Renderer:
    """Renderer, include/renderer.h:77-119."""

    kind = RENDERER_PERFORMANCE

    def __init__(self, scene_info, occupancy_grid, nerf_network: NerfNetwork):
        self._scene_info = scene_info
        self._occupancy_grid = occupancy_grid
        self._nerf_network = nerf_network
        h = C.c_void_p()
        L.check(L.load().fvc_renderer_create(nerf_network.handle, self.kind, C.byref(h)))
        self.handle = h

    def resizeRenderbuffers(self, resolution) -> None:
        L.check(L.load().fvc_renderer_resize(self.handle, int(resolution[0]), int(resolution[1])))

    def set_stream(self, stream_handle: int | None) -> None:
        L.check(L.load().fvc_renderer_set_stream(self.handle, stream_handle))

    def set_network_path(self, use_tcgen05: bool) -> None:
        """tcgen05 (default) or mma.sync network kernels."""
        L.check(L.load().fvc_renderer_set_network_path(self.handle, int(bool(use_tcgen05))))

    def set_build_network_path(self, use_tcgen05: bool) -> None:
        """The cache builds' density network: mma.sync (default, faster here) or tcgen05; same slots."""
        L.check(L.load().fvc_renderer_set_build_network_path(self.handle, int(bool(use_tcgen05))))

    def set_empty_space_skipping(self, on: bool) -> None:
        """Occupancy lookups once per empty cell (default) or every step; identical results."""
        L.check(L.load().fvc_renderer_set_empty_space_skipping(self.handle, int(bool(on))))

    def set_fused_classify(self, on: bool) -> None:
        """Cache renderers: classification inside the march + one network launch (default) or the separate pass."""
        L.check(L.load().fvc_renderer_set_fused_classify(self.handle, int(bool(on))))

    def set_tiling(self, m_tile: int = 128, batch_rows: int = 0) -> None:
        """tcgen05 network tile height (64, 128, 256) and compaction batch (rows per sub-iteration, 0 = capacity)."""
        L.check(L.load().fvc_renderer_set_tiling(self.handle, int(m_tile), int(batch_rows)))

    FP16, BF16, FP8_E4M3 = 0, 1, 2

    def set_precision(self, precision: int) -> None:
        """MLP precision of the plain tcgen05 path: FP16 (default), BF16 or FP8_E4M3."""
        L.check(L.load().fvc_renderer_set_precision(self.handle, int(precision)))

    def set_kernel_timing(self, enable: bool) -> None:
        """CUDA-event timing of each resample network launch (see _render_stats.timed_kernel_ms)."""
        L.check(L.load().fvc_renderer_set_kernel_timing(self.handle, int(bool(enable))))

    def set_max_samples_per_ray(self, n: int) -> None:
        L.check(L.load().fvc_renderer_set_max_samples_per_ray(self.handle, n))

    def render(self, rm_info: L.RaymarchInfo, render_buffer: RenderBuffer, debug_data=None) -> None:
        """render(RaymarchInfo, RenderBuffer&) with host buffers (synchronous)."""
        out = render_buffer.outputs()
        L.check(L.load().fvc_render(self.handle, C.byref(rm_info), C.byref(out)))

    def render_device(self, rm_info: L.RaymarchInfo, image=None, results=None, ray_counts=None, contrib_resample=None,
                      contrib_cache=None) -> None:
        """Enqueue a render into device buffers (pointers or torch tensors); cache renderers add the
        per-pixel contribution weights of resampled and cache samples to contrib_* (float, W x H)."""
        out = L.RenderOutputs()
        out.image_rgba8, out.results, out.ray_counts = L.ptr(image), L.ptr(results), L.ptr(ray_counts)
        out.contrib_resample, out.contrib_cache = L.ptr(contrib_resample), L.ptr(contrib_cache)
        L.check(L.load().fvc_render_device(self.handle, C.byref(rm_info), C.byref(out)))

    def render_backward(self, rm_info: L.RaymarchInfo, pixels, target, grads: "Gradients", pred=None, n_rays=None) -> float:
        """Forward + adjoint of the plain render at device `pixels` (int32 y*W+x)
        against device `target` [n,3]: adds dL/dparam to `grads`, returns the
        mean squared error L; `pred` (device [n,4]) receives (C, T)."""
        n = int(n_rays if n_rays is not None else pixels.numel())
        loss = C.c_double()
        L.check(L.load().fvc_render_backward(self.handle, grads.handle, C.byref(rm_info), L.ptr(pixels), n, L.ptr(target),
                                             C.byref(loss), L.ptr(pred)))
        return loss.value

    @staticmethod
    def _batch_args(infos, image, results, ray_counts):
        arr = (L.RaymarchInfo * len(infos))(*infos)
        out = L.RenderOutputs()
        out.image_rgba8, out.results, out.ray_counts = L.ptr(image), L.ptr(results), L.ptr(ray_counts)
        return arr, out

    def render_batch(self, infos, image=None, results=None, ray_counts=None) -> None:
        """Render several views in one CUDA-graph launch into device buffers
        holding the views back to back (asynchronous on the renderer's stream)."""
        arr, out = self._batch_args(infos, image, results, ray_counts)
        L.check(L.load().fvc_render_batch(self.handle, arr, len(infos), C.byref(out)))

    def render_batch_cached(self, infos, caches, image=None, results=None, ray_counts=None) -> None:
        """Cache renderers: view v renders against its own built cache caches[v]."""
        arr, out = self._batch_args(infos, image, results, ray_counts)
        handles = (C.c_void_p * len(caches))(*[c.handle.value for c in caches])
        L.check(L.load().fvc_render_batch_cached(self.handle, arr, len(infos), handles, C.byref(out)))

    def set_autotune_space(self, m_tiles, batch_rows, march_steps) -> None:
        """Candidate network tiles (32 = mma.sync), compaction batches and march lengths of autotune()."""
        arr = lambda v: (C.c_int * len(v))(*[int(x) for x in v])  # noqa: E731
        L.check(L.load().fvc_renderer_set_autotune_space(self.handle, arr(m_tiles), len(m_tiles), arr(batch_rows), len(batch_rows),
                                                         arr(march_steps), len(march_steps)))

    def autotune(self, infos, image=None, results=None, ray_counts=None) -> L.AutotuneResult:
        """Pick the network tile and marching batch that render this batch fastest."""
        arr, out = self._batch_args(infos, image, results, ray_counts)
        res = L.AutotuneResult()
        L.check(L.load().fvc_renderer_autotune(self.handle, arr, len(infos), C.byref(out), C.byref(res)))
        return res

    def synchronize(self) -> None:
        L.check(L.load().fvc_renderer_synchronize(self.handle))

    @property
    def _render_stats(self) -> L.RenderStats:
        s = L.RenderStats()
        L.check(L.load().fvc_render_stats(self.handle, C.byref(s)))
        return s

    def __del__(self):
        if getattr(self, "handle", None) and L._lib is not None:
            L._lib.fvc_renderer_destroy(self.handle)
            self.handle = None


class BasicRenderer(Renderer):
    """BasicRenderer, include/basic_renderer.h (same method as PerformanceRenderer)."""
    kind = RENDERER_BASIC


class PerformanceRenderer(Renderer):
    """PerformanceRenderer, include/performance_renderer.h:19-64."""
    kind = RENDERER_PERFORMANCE


class Gradients:
    """fp32 gradients of a model's parameters in the model file layouts:
    hash table [entries, 2], density-MLP blob, color-head blob (fvc_grad)."""

    def __init__(self, nerf_network: NerfNetwork):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.fvc_grad_create(nerf_network.handle, C.byref(h)))
        self.handle = h
        self._net = nerf_network
        a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
        L.check(lib.fvc_grad_sizes(h, C.byref(a), C.byref(b), C.byref(c)))
        self.sizes = (a.value, b.value, c.value)

    def zero(self) -> None:
        L.check(L.load().fvc_grad_zero(self.handle))

    def cache_latents(self) -> np.ndarray:
        """Gradients of the cache brick latents [slots, 512, 8] (cached backward)."""
        n = C.c_size_t()
        L.check(L.load().fvc_grad_cache_latents(self.handle, None, C.byref(n)))
        out = np.zeros(n.value, np.float32)
        if n.value:
            L.check(L.load().fvc_grad_cache_latents(self.handle, L.ptr(out), C.byref(n)))
        return out.reshape(-1, 512, 8)

    def read(self):
        t, b, h = (np.zeros(n, np.float32) for n in self.sizes)
        L.check(L.load().fvc_grad_read(self.handle, L.ptr(t), L.ptr(b), L.ptr(h)))
        return t, b, h

    def __del__(self):
        if getattr(self, "handle", None) and L._lib is not None:
            L._lib.fvc_grad_destroy(self.handle)
            self.handle = None


class Cache:
    """Cache, include/cache.h:12-74 (device storage owned by the library)."""

    def __init__(self):
        h = C.c_void_p()
        L.check(L.load().fvc_cache_create(C.byref(h)))
        self.handle = h

    def dims(self):
        f, b, d = L.Int3(), L.Int3(), L.Int3()
        L.check(L.load().fvc_cache_dims(self.handle, C.byref(f), C.byref(b), C.byref(d)))
        return (f.x, f.y, f.z), (b.x, b.y, b.z), (d.x, d.y, d.z)

    def read(self, voxels: bool = True):
        """packed brick index [bZ,bY,bX], known ranges [H,W], voxels [slots,512,8] u32 words."""
        lib = L.load()
        nb, nk, nv = C.c_size_t(), C.c_size_t(), C.c_size_t()
        L.check(lib.fvc_cache_read(self.handle, None, C.byref(nb), None, C.byref(nk), None, C.byref(nv)))
        (fW, fH, fD), (bX, bY, bZ), _ = self.dims()
        packed = np.zeros(nb.value, np.int32)
        known = np.zeros(nk.value, np.float32)
        vox = np.zeros(nv.value, np.uint32) if voxels else None
        L.check(lib.fvc_cache_read(self.handle, L.ptr(packed), None, L.ptr(known), None, L.ptr(vox), None))
        return packed.reshape(bZ, bY, bX), known.reshape(fH, fW), (vox.reshape(-1, 512, 8) if voxels else None)

    def __del__(self):
        if getattr(self, "handle", None) and L._lib is not None:
            L._lib.fvc_cache_destroy(self.handle)
            self.handle = None


class CachePerformanceRenderer(Renderer):
    """CachePerformanceRenderer, include/cache_performance_renderer.h:21-131,
    with CacheRenderer's cache control (include/cache_renderer.h:34-109)."""

    kind = RENDERER_CACHE_PERFORMANCE
    ONLY_CACHE, ONLY_RESAMPLED, DEFAULT = 1, 2, 0

    def __init__(self, scene_info, occupancy_grid, nerf_network, cache: Cache, next_cache: Cache):
        super().__init__(scene_info, occupancy_grid, nerf_network)
        self._cache, self._cache_next = cache, next_cache
        L.check(L.load().fvc_renderer_set_caches(self.handle, cache.handle, next_cache.handle))

    def attach_caches(self, cache: Cache, next_cache: Cache) -> None:
        """Render from `cache`, build into `next_cache` (the constructor's pair)."""
        L.check(L.load().fvc_renderer_set_caches(self.handle, cache.handle, next_cache.handle))
        self._cache, self._cache_next = cache, next_cache

    def set_cache_sizing(self, est_samples_per_ray: int = 32, brick_sparsity: float = 0.5) -> None:
        """resizeCache's two estimates (the reference's compile-time 32 and 0.5); takes effect at the next resizeCache."""
        L.check(L.load().fvc_cache_set_sizing(self.handle, int(est_samples_per_ray), float(brick_sparsity)))

    def resizeCache(self, resolution, stepsize_info) -> None:
        L.check(L.load().fvc_cache_resize(self.handle, int(resolution[0]), int(resolution[1]), C.byref(stepsize_info)))

    def initCacheBlockwise(self, rm_info: L.RaymarchInfo, debug_image_buffer=None) -> None:
        L.check(L.load().fvc_cache_build(self.handle, C.byref(rm_info)))

    def initCache(self, rm_info: L.RaymarchInfo, debug_image_buffer=None) -> None:
        """The per-ray fill (CacheRenderer::initCache, src/cache_renderer.cu:848-928)."""
        L.check(L.load().fvc_cache_build_per_ray(self.handle, C.byref(rm_info)))

    def swapCache(self) -> None:
        L.check(L.load().fvc_cache_swap(self.handle))
        self._cache, self._cache_next = self._cache_next, self._cache

    def setCacheSettings(self, settings: L.CacheSettings) -> None:
        L.check(L.load().fvc_renderer_set_cache_settings(self.handle, C.byref(settings)))

    def set_render_mode(self, mode: int) -> None:
        L.check(L.load().fvc_renderer_set_render_mode(self.handle, mode))

    @property
    def _init_stats(self) -> L.CacheStats:
        s = L.CacheStats()
        L.check(L.load().fvc_cache_stats(self.handle, C.byref(s)))
        return s


class CacheBasicRenderer(CachePerformanceRenderer):
    """CacheBasicRenderer, include/cache_basic_renderer.h:10-40: the cached
    render with the basic renderer's per-sample semantics (every CacheSettings
    field applies; a cache sample composites with its looked-up density)."""

    kind = RENDERER_CACHE_BASIC


def change_sampling_rate(stepsize_info: L.StepsizeInfo, factor: float, scene_info: L.SceneInfo) -> L.StepsizeInfo:
    """StepsizeInfo::changeSamplingRate (include/common.h:130-135) on a copy:
    cone angle and step size divided by ``factor``, derived fields refilled
    (setAdditionalInfo, include/common.h:109-131)."""
    s = L.StepsizeInfo.from_buffer_copy(stepsize_info)
    s.cone_angle /= factor
    s.stepsize /= factor
    L.check(L.load().fvc_stepsize_setup(C.byref(scene_info), C.byref(s)))
    return s


# DensityInterpolVariant and InterpolFunction (include/cache_renderer.h:14-22, include/common.h:221-227)
DENSITY, ALPHA, INTERMEDIATES, DENSITY_INTERMEDIATES, ALPHA_INTERMEDIATES = range(5)
LINEAR, SMOOTHSTEP, SMOOTHERSTEP, NEAREST = range(4)


def default_cache_settings(interpol_variant: int = DENSITY, interpol_function: int = LINEAR) -> L.CacheSettings:
    """CacheRenderer::default_cache_settings, include/cache_renderer.h:55-63,
    optionally with another variant / interpolation function."""
    s = L.CacheSettings()
    s.interpol_variant, s.interpol_function = interpol_variant, interpol_function
    s.use_hw_interpol = s.reweight_intermediates = s.disable_reweighting_first_intermediate = 1
    s.use_inter_brick_interpolation = 1
    return s


def eval_cache_settings(loader) -> L.CacheSettings:
    """The settings eval gives the cache renderer (src/eval.cu:215-222):
    DensityIntermediates for a model whose first latent is the density,
    else Density; Linear interpolation."""
    fld = bool(loader.nerf_network.properties()["first_latent_is_density"])
    return default_cache_settings(DENSITY_INTERMEDIATES if fld else DENSITY, LINEAR)


__all__ = ["load_data", "LoaderData", "NerfNetwork", "Renderer", "BasicRenderer", "PerformanceRenderer", "Cache", "Gradients",
           "CachePerformanceRenderer", "CacheBasicRenderer", "RenderBuffer", "raymarch_info", "camera_info", "camera_dict",
           "default_cache_settings", "eval_cache_settings", "change_sampling_rate", "DENSITY", "ALPHA", "INTERMEDIATES", "DENSITY_INTERMEDIATES",
           "ALPHA_INTERMEDIATES", "LINEAR", "SMOOTHSTEP", "SMOOTHERSTEP", "NEAREST"]
