"""ctypes binding of the CPU oracle (fvc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg as the checker.  The product package never
imports it.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfvc_oracle.so")

F3 = C.c_float * 3


class OrcScene(C.Structure):
    _fields_ = [("grid_nlvl", C.c_int), ("normalized", C.c_int), ("contraction", C.c_int), ("is_open_gl", C.c_int),
                ("aabb_from", F3), ("aabb_to", F3), ("c_from", F3), ("c_to", F3), ("alpha_thre", C.c_float)]


class OrcSteps(C.Structure):
    _fields_ = [(n, C.c_float) for n in ["cone_angle", "log1p_c", "stepsize", "near_", "near_i", "far_", "dt_min",
                                         "dt_max", "t_min", "t_max", "i_min", "i_max", "log1p_c_lo"]] + [("use_libm", C.c_int)]


class OrcCam(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("is_open_gl", C.c_int), ("fx", C.c_float), ("fy", C.c_float),
                ("px", C.c_float), ("py", C.c_float), ("c2w", C.c_float * 12), ("w2c", C.c_float * 12),
                ("nd", C.c_int), ("motion_blur", C.c_int), ("sample_index", C.c_int), ("aperature", C.c_float),
                ("focus_z", C.c_float), ("nc2w", C.c_float * 12)]


class OrcNet(C.Structure):
    _fields_ = [("n_levels", C.c_int), ("F", C.c_int), ("scale", C.c_float * 32), ("res", C.c_uint32 * 32),
                ("size", C.c_uint32 * 32), ("offset", C.c_uint32 * 32), ("dense", C.c_uint32 * 32),
                ("table", C.c_void_p), ("width", C.c_int), ("enc_w", C.c_int), ("enc_w_pad", C.c_int),
                ("base_out_pad", C.c_int), ("base_w", C.c_void_p), ("head_layers", C.c_int), ("head_in", C.c_int),
                ("head_in_pad", C.c_int), ("n_latents", C.c_int), ("latent_offset", C.c_int), ("head_w", C.c_void_p),
                ("mimic_fp16", C.c_int), ("view_dependent", C.c_int), ("first_w", C.c_void_p), ("freq_deg", C.c_int)]


class OrcCacheDims(C.Structure):
    _fields_ = [(n, C.c_int) for n in ["fW", "fH", "fD", "bX", "bY", "bZ", "dX", "dY", "dZ"]]


class OrcCache(C.Structure):
    _fields_ = [("dims", OrcCacheDims), ("packed_index", C.c_void_p), ("known_ranges", C.c_void_p),
                ("vox_density", C.c_void_p), ("vox_isset", C.c_void_p), ("vox_latents", C.c_void_p),
                ("n_bricks_set", C.c_int), ("n_demanded", C.c_int), ("n_iterations", C.c_int),
                ("n_samples", C.c_longlong), ("slot_of_brick_order", C.c_void_p), ("variant", C.c_int), ("interp", C.c_int),
                ("basic", C.c_int), ("reweight", C.c_int), ("keep_first", C.c_int), ("inter_brick", C.c_int)]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "fvc_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", HERE, "_build/libfvc_oracle.so"], check=True, capture_output=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P = C.POINTER
        _lib.orc_setup_steps.argtypes = [P(OrcScene), P(OrcSteps)]
        _lib.orc_grid_to_morton_bits.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_trace_ray.argtypes = [P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, C.c_int, C.c_int, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_trace_ray.restype = C.c_int
        _lib.orc_step_from_t.argtypes = [P(OrcSteps), C.c_float]
        _lib.orc_step_from_t.restype = C.c_float
        _lib.orc_smp_sobol.argtypes = [C.c_uint32, C.c_uint32]
        _lib.orc_smp_sobol.restype = C.c_uint32
        _lib.orc_smp_ld_val.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        _lib.orc_smp_ld_val.restype = C.c_float
        _lib.orc_smp_pixel_offset.argtypes = [C.c_uint32, C.c_void_p]
        _lib.orc_smp_t_offset.argtypes = [C.c_uint32, C.c_uint32]
        _lib.orc_smp_t_offset.restype = C.c_float
        _lib.orc_smp_square_to_disk.argtypes = [C.c_float, C.c_float, C.c_void_p]
        _lib.orc_smp_camera_slerp.argtypes = [C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
        _lib.orc_generate_ray.argtypes = [P(OrcScene), P(OrcSteps), P(OrcCam), C.c_int, C.c_int, C.c_void_p]
        _lib.orc_t_from_step.argtypes = [P(OrcSteps), C.c_float]
        _lib.orc_t_from_step.restype = C.c_float
        _lib.orc_occupied.argtypes = [P(OrcScene), C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_contract.argtypes = [P(OrcScene), C.c_void_p, C.c_void_p]
        _lib.orc_logf.argtypes = [C.c_float]
        _lib.orc_logf.restype = C.c_float
        _lib.orc_expf.argtypes = [C.c_float]
        _lib.orc_expf.restype = C.c_float
        _lib.orc_inference.argtypes = [P(OrcNet), C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        _lib.orc_hash_encode.argtypes = [P(OrcNet), C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_base_outputs.argtypes = [P(OrcNet), C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        _lib.orc_render_plain.argtypes = [P(OrcNet), P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, C.c_int, C.c_int,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        _lib.orc_loss_grad.argtypes = [P(OrcNet), P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_int, C.c_void_p]
        _lib.orc_loss_grad.restype = C.c_double
        _lib.orc_loss_grad_cached.argtypes = [P(OrcNet), P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, P(OrcCache),
                                              P(OrcCam), P(OrcSteps), C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                              C.c_void_p]
        _lib.orc_loss_grad_cached.restype = C.c_double
        _lib.orc_composite_rows.argtypes = [C.c_int, C.c_int, P(OrcSteps), C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p]
        _lib.orc_cache_dims.argtypes = [P(OrcScene), P(OrcSteps), C.c_int, C.c_int, P(OrcCacheDims)]
        _lib.orc_cache_build.argtypes = [P(OrcNet), P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, P(OrcCache), C.c_int]
        _lib.orc_cache_build_per_ray.argtypes = [P(OrcNet), P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, P(OrcCache),
                                                 C.c_int]
        _lib.orc_render_cached.argtypes = [P(OrcNet), P(OrcScene), P(OrcSteps), P(OrcCam), C.c_void_p, P(OrcCache),
                                           P(OrcCam), P(OrcSteps), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_int, C.c_void_p, C.c_void_p]
    return _lib


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


def make_scene(cfg_scene: dict) -> OrcScene:
    s = OrcScene()
    s.grid_nlvl = int(cfg_scene["grid_nlvl"])
    s.normalized = int(bool(cfg_scene.get("normalized", False)))  # nerfacc exports: false; .ingp snapshots: true
    a = cfg_scene["aabb"]
    s.aabb_from[:] = a[:3]
    s.aabb_to[:] = a[3:]
    if "contraction" in cfg_scene and "aabb" in cfg_scene["contraction"]:
        s.contraction = 3
        ca = cfg_scene["contraction"]["aabb"]
        s.c_from[:] = ca[:3]
        s.c_to[:] = ca[3:]
    else:
        s.contraction = 1
    s.is_open_gl = int(bool(cfg_scene.get("is_open_gl", False)))
    s.alpha_thre = float(cfg_scene["alpha_thre"])
    return s


def make_steps(scene: OrcScene, cone: float, stepsize: float, near: float, far: float, use_libm: bool = False) -> OrcSteps:
    st = OrcSteps()
    st.cone_angle, st.stepsize, st.near_, st.far_ = cone, stepsize, near, far
    st.use_libm = int(use_libm)
    lib().orc_setup_steps(C.byref(scene), C.byref(st))
    return st


def make_cam(cam: dict) -> OrcCam:
    c = OrcCam()
    c.W, c.H = cam["resolution"]
    c.is_open_gl = int(bool(cam["is_open_gl"]))
    c.fx, c.fy = cam["focal"]
    c.px, c.py = cam["principal"]
    c.c2w[:] = np.asarray(cam["cam2world"], np.float32).ravel().tolist()
    c.w2c[:] = np.asarray(cam["world2cam"], np.float32).ravel().tolist()
    # RaymarchInfo's sampling fields (camera dict keys of frustumvolumecaching_gb300.raymarch_info)
    c.nd = int(not cam.get("deterministic", True))
    c.motion_blur = int(bool(cam.get("motion_blur", False)))
    c.sample_index = int(cam.get("sample_index", 0))
    c.aperature = float(cam.get("aperature", 0.0))
    c.focus_z = float(cam.get("focus_z", 1.0))
    c.nc2w[:] = np.asarray(cam.get("next_cam2world", cam["cam2world"]), np.float32).ravel().tolist()
    return c


class OracleModel:
    """A nerfacc-format export held for the oracle (parsed independently of
    the product's C++ loader)."""

    def __init__(self, model_dir: str, mimic_fp16: bool = False, use_libm: bool = False):
        from frustumvolumecaching_gb300.model import hash_grid_levels
        with open(os.path.join(model_dir, "config.json")) as f:
            cfg = json.load(f)
        self.cfg = cfg
        sc = cfg["scene"]
        self.scene = make_scene(sc)
        self.steps = make_steps(self.scene, sc["cone_angle"], sc["stepsize"], sc["near"], sc["far"], use_libm)
        enc = cfg["mlp_base"]["encoding"]
        self.levels = hash_grid_levels(enc["n_levels"], enc["base_resolution"], enc["per_level_scale"],
                                       enc["log2_hashmap_size"], enc.get("fvc_level_scales"))
        F = enc["n_features_per_level"]
        self.table = np.fromfile(os.path.join(model_dir, "pos_enc.dat"), np.uint16)
        n_entries = self.levels[-1].offset + self.levels[-1].size
        assert self.table.size == n_entries * F, "pos_enc.dat size does not match the hash-grid layout"
        width = cfg["mlp_base"]["network"]["n_neurons"]
        enc_w = enc["n_levels"] * F
        enc_w_pad = (enc_w + 15) // 16 * 16
        n_out = cfg["mlp_base"]["n_output"]
        base_out_pad = (n_out + 15) // 16 * 16
        self.base_w = np.fromfile(os.path.join(model_dir, "mlp_base.dat"), np.uint16)
        assert self.base_w.size == width * enc_w_pad + base_out_pad * width
        head = cfg["mlp_head"]
        n_hidden = head["network"]["n_hidden_layers"]
        # the view-dependent split network (NerfNetwork::init_viewdep, include/nerf_network.h:120-158)
        first = cfg.get("mlp_first_head")
        self.view_dependent = first is not None
        if first is not None:
            first_lat_dens = bool(first.get("first_latent_is_density", True))
            n_lat = int(first["n_output"])
            head_in = int(head.get("n_input", 32 + n_lat))
            self.first_w = np.fromfile(os.path.join(model_dir, "mlp_first_head.dat"), np.uint16)
            assert self.first_w.size == width * 32 + 16 * width
        else:
            first_lat_dens = bool(head.get("first_latent_is_density", True))
            n_lat = int(head.get("n_latents", n_out))
            head_in = int(head.get("n_input", 16 + n_lat))
            self.first_w = np.zeros(1, np.uint16)
        head_in_pad = (head_in + 15) // 16 * 16
        self.head_w = np.fromfile(os.path.join(model_dir, "mlp_head.dat"), np.uint16)
        assert self.head_w.size == width * head_in_pad + (n_hidden - 1) * width * width + 16 * width
        grid = np.fromfile(os.path.join(model_dir, "occupancy_grid.dat"), np.uint8)
        self.grid = grid
        self.bits = np.zeros(grid.size // 8, np.uint8)
        lib().orc_grid_to_morton_bits(ptr(grid), self.scene.grid_nlvl, ptr(self.bits))
        n = OrcNet()
        n.n_levels, n.F = enc["n_levels"], F
        for i, lv in enumerate(self.levels):
            n.scale[i], n.res[i], n.size[i], n.offset[i], n.dense[i] = lv.scale, lv.res, lv.size, lv.offset, int(lv.dense)
        n.table = ptr(self.table)
        n.width, n.enc_w, n.enc_w_pad, n.base_out_pad = width, enc_w, enc_w_pad, base_out_pad
        n.base_w = ptr(self.base_w)
        n.head_layers = n_hidden + 1
        n.head_in, n.head_in_pad, n.n_latents = head_in, head_in_pad, n_lat
        n.latent_offset = 0 if first_lat_dens else 1
        n.head_w = ptr(self.head_w)
        n.mimic_fp16 = int(mimic_fp16)
        n.view_dependent = int(self.view_dependent)
        n.first_w = ptr(self.first_w)
        n.freq_deg = int(head.get("freq_encoding_degree", 0))
        self.net = n

    # -- evaluation --------------------------------------------------------
    def inference(self, pos: np.ndarray, dir01: np.ndarray, threads: int | None = None) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float32)
        dir01 = np.ascontiguousarray(dir01, np.float32)
        out = np.zeros((pos.shape[0], 4), np.float64)
        lib().orc_inference(C.byref(self.net), ptr(pos), ptr(dir01), pos.shape[0], ptr(out), threads or default_threads())
        return out

    def base_outputs(self, pos: np.ndarray, dir01: np.ndarray, threads: int | None = None) -> np.ndarray:
        """The density network's padded outputs (float64, row 0 the log-density) at contracted positions."""
        pos = np.ascontiguousarray(pos, np.float32)
        dir01 = np.ascontiguousarray(dir01, np.float32)
        out = np.zeros((pos.shape[0], self.net.base_out_pad), np.float64)
        lib().orc_base_outputs(C.byref(self.net), ptr(pos), ptr(dir01), pos.shape[0], ptr(out), threads or default_threads())
        return out

    def hash_encode(self, pos: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float32)
        out = np.zeros((pos.shape[0], self.net.enc_w_pad), np.float64)
        lib().orc_hash_encode(C.byref(self.net), ptr(pos), pos.shape[0], ptr(out))
        return out

    def render_plain(self, cam: dict, rows: tuple[int, int] | None = None, threads: int | None = None):
        c = make_cam(cam)
        W, H = c.W, c.H
        r0, r1 = rows or (0, H)
        res = np.zeros((H, W, 4), np.float32)
        ns = np.zeros((H, W), np.int32)
        nst = np.zeros((H, W), np.int32)
        lib().orc_render_plain(C.byref(self.net), C.byref(self.scene), C.byref(self.steps), C.byref(c), ptr(self.bits),
                               r0, r1, ptr(res), ptr(ns), ptr(nst), threads or default_threads())
        return res, ns, nst

    # -- differentiable render --------------------------------------------
    def loss_grad(self, cam: dict, pixels: np.ndarray, target: np.ndarray, grads: bool = True,
                  perturb=None, threads: int | None = None):
        """Loss of the plain render at `pixels` (y*W+x) against target [n,3]
        and, if grads, the float64 gradients (table, base blob, head blob).
        perturb = (groups, indices, deltas) added to the parameters first.
        Returns (loss, g_table, g_base, g_head, pred[n,4])."""
        c = make_cam(cam)
        px = np.ascontiguousarray(pixels, np.int32)
        tg = np.ascontiguousarray(target, np.float32).reshape(-1)
        pred = np.zeros((px.size, 4), np.float64)
        gt = np.zeros(self.table.size, np.float64) if grads else None
        gb = np.zeros(self.base_w.size, np.float64) if grads else None
        gh = np.zeros(self.head_w.size, np.float64) if grads else None
        if perturb is not None:
            pg = np.ascontiguousarray(perturb[0], np.int32)
            pi = np.ascontiguousarray(perturb[1], np.int64)
            pd = np.ascontiguousarray(perturb[2], np.float64)
            npert, pgp, pip, pdp = pg.size, ptr(pg), ptr(pi), ptr(pd)
        else:
            npert, pgp, pip, pdp = 0, None, None, None
        loss = lib().orc_loss_grad(C.byref(self.net), C.byref(self.scene), C.byref(self.steps), C.byref(c), ptr(self.bits),
                                   ptr(px), px.size, ptr(tg), ptr(gt) if grads else None, ptr(gb) if grads else None,
                                   ptr(gh) if grads else None, pgp, pip, pdp, npert, threads or default_threads(), ptr(pred))
        return loss, gt, gb, gh, pred

    def cache_dims(self, W: int, H: int, steps: OrcSteps | None = None, sizing: tuple[int, float] = (32, 0.5)) -> OrcCacheDims:
        """Cache dimensions of resizeCache (src/cache_renderer.cu:832-846); `sizing` = (estimated samples
        per ray, brick sparsity), the reference's compile-time (32, 0.5) by default."""
        d = OrcCacheDims()
        lib().orc_cache_dims(C.byref(self.scene), C.byref(steps or self.steps), W, H, C.byref(d))
        if tuple(sizing) != (32, 0.5):
            est_bricks = (W * H * int(sizing[0])) // max(1, int(np.float32(sizing[1]) * np.float32(512.0)))
            d.dZ = max(1, (est_bricks + d.dX * d.dY - 1) // (d.dX * d.dY))
        return d

    def cache_build(self, cam: dict, threads: int | None = None, variant: int = 0, interp: int = 0,
                    steps: OrcSteps | None = None) -> "OracleCache":
        """Blockwise build; `variant` / `interp` are CacheSettings'
        interpol_variant and interpol_function (the latter used by lookups
        through the returned cache; change `cache.s.interp` to render with
        another); `steps` the cache's StepsizeInfo (default: the model's)."""
        c = make_cam(cam)
        st = steps or self.steps
        cc = OracleCache(self.cache_dims(c.W, c.H, st), cam)
        cc.steps = st
        cc.s.variant, cc.s.interp = variant, interp
        lib().orc_cache_build(C.byref(self.net), C.byref(self.scene), C.byref(st), C.byref(c), ptr(self.bits),
                              C.byref(cc.s), threads or default_threads())
        return cc

    def cache_build_per_ray(self, cam: dict, threads: int | None = None, variant: int = 0) -> "OracleCache":
        """The per-ray fill (CacheRenderer::initCache) with the model's steps."""
        c = make_cam(cam)
        cc = OracleCache(self.cache_dims(c.W, c.H), cam)
        cc.s.variant = variant
        lib().orc_cache_build_per_ray(C.byref(self.net), C.byref(self.scene), C.byref(self.steps), C.byref(c), ptr(self.bits),
                                      C.byref(cc.s), threads or default_threads())
        return cc

    def loss_grad_cached(self, cam: dict, cache: "OracleCache", pixels: np.ndarray, target: np.ndarray, grads: bool = True,
                         perturb=None, threads: int | None = None):
        """Cached-render loss at `pixels` against target [n,3] and, if grads, the
        float64 gradients (table, base blob, head blob, voxel latents
        [slots*512*8]).  perturb = (latent indices, deltas)."""
        c = make_cam(cam)
        cc = make_cam(cache.cam)
        px = np.ascontiguousarray(pixels, np.int32)
        tg = np.ascontiguousarray(target, np.float32).reshape(-1)
        pred = np.zeros((px.size, 4), np.float64)
        outs = [np.zeros(n, np.float64) if grads else None
                for n in (self.table.size, self.base_w.size, self.head_w.size, cache.vox_latents.size)]
        if perturb is not None:
            pi = np.ascontiguousarray(perturb[0], np.int64)
            pd = np.ascontiguousarray(perturb[1], np.float64)
            npert, pip, pdp = pi.size, ptr(pi), ptr(pd)
        else:
            npert, pip, pdp = 0, None, None
        loss = lib().orc_loss_grad_cached(C.byref(self.net), C.byref(self.scene), C.byref(self.steps), C.byref(c),
                                          ptr(self.bits), C.byref(cache.s), C.byref(cc), C.byref(self.steps), ptr(px), px.size,
                                          ptr(tg), *[ptr(o) if o is not None else None for o in outs], pip, pdp, npert,
                                          threads or default_threads(), ptr(pred))
        return (loss, *outs, pred)

    # why samples were not cache hits (orc_render_cached's reasons[1..7])
    REASONS = ("outside_fov", "outside_depth", "before_near", "beyond_known", "brick_unset", "voxel_empty", "alpha")

    def render_cached(self, cam: dict, cache: "OracleCache", mode: int = 0, rows=None, threads: int | None = None,
                      reasons: bool = False, contrib: bool = False):
        """(results, counts), plus {reason: samples} with reasons=True, plus the per-pixel contribution
        weights [H, W, 2] (resampled, cache; alpha T summed) with contrib=True."""
        c = make_cam(cam)
        cc = make_cam(cache.cam)
        W, H = c.W, c.H
        r0, r1 = rows or (0, H)
        res = np.zeros((H, W, 4), np.float32)
        counts = np.zeros((H, W, 4), np.int32)
        why = np.zeros(8, np.int64)
        con = np.zeros((H, W, 2), np.float64) if contrib else None
        lib().orc_render_cached(C.byref(self.net), C.byref(self.scene), C.byref(self.steps), C.byref(c), ptr(self.bits),
                                C.byref(cache.s), C.byref(cc), C.byref(cache.steps or self.steps), mode, r0, r1, ptr(res),
                                ptr(counts), threads or default_threads(), ptr(why), ptr(con) if contrib else None)
        out = (res, counts)
        if reasons:
            out += ({k: int(why[i + 1]) for i, k in enumerate(self.REASONS)},)
        if contrib:
            out += (con,)
        return out


class OracleCache:
    def __init__(self, dims: OrcCacheDims, cam: dict):
        self.cam = cam
        self.dims = dims
        self.steps = None  # the StepsizeInfo the cache was built with (None: the model's)
        self.settings = None  # set below, once the ctypes struct exists
        nb = dims.bX * dims.bY * dims.bZ
        slots = dims.dX * dims.dY * dims.dZ
        self.packed_index = np.full(nb, -1, np.int32)
        self.known_ranges = np.zeros(dims.fW * dims.fH, np.float32)
        self.vox_density = np.zeros(slots * 512, np.float32)
        self.vox_isset = np.zeros(slots * 512, np.float32)
        self.vox_latents = np.zeros(slots * 512 * 8, np.uint16)
        s = OrcCache()
        s.dims = dims
        s.packed_index, s.known_ranges = ptr(self.packed_index), ptr(self.known_ranges)
        s.vox_density, s.vox_isset, s.vox_latents = ptr(self.vox_density), ptr(self.vox_isset), ptr(self.vox_latents)
        s.slot_of_brick_order = None
        s.reweight = s.keep_first = s.inter_brick = 1  # CacheRenderer::default_cache_settings
        self.s = s

    def render_as_basic(self, variant: int = 0, interp: int = 0, reweight: bool = True, keep_first: bool = True,
                        inter_brick: bool = True) -> "OracleCache":
        """Look up with CacheBasicRenderer's semantics and these settings."""
        self.s.basic, self.s.variant, self.s.interp = 1, variant, interp
        self.s.reweight, self.s.keep_first, self.s.inter_brick = int(reweight), int(keep_first), int(inter_brick)
        return self

    def load_device_cache(self, packed: np.ndarray, known: np.ndarray, voxels: np.ndarray) -> None:
        """Use a device-built cache (fvc_cache_read: packed index, known ranges,
        voxels as [slots, 512, 8] u32 words: density f32, isset f32, 2 pad,
        8 fp16 latents) instead of the oracle's own build."""
        self.packed_index[:] = packed.reshape(-1)
        self.known_ranges[:] = known.reshape(-1)
        v = voxels.reshape(-1, 8)
        n = min(v.shape[0], self.vox_density.size)
        self.vox_density[:n] = v[:n, 0].view(np.float32)
        self.vox_isset[:n] = v[:n, 1].view(np.float32)
        self.vox_latents[:n * 8] = np.ascontiguousarray(v[:n, 4:8]).view(np.uint16).reshape(-1)

    @property
    def n_bricks_set(self):
        return self.s.n_bricks_set

    @property
    def n_demanded(self):
        return self.s.n_demanded

    @property
    def n_samples(self):
        return self.s.n_samples


def composite_image(results: np.ndarray, sample_index: int = 0, prev: np.ndarray | None = None) -> np.ndarray:
    """writeImageBuffer_performance_kernel (src/performance_renderer.cu:127-149):
    white background, int(c*256) clamped to [0,255], progressive average."""
    rgb = results[..., :3] + results[..., 3:4]
    if prev is not None and sample_index > 0:
        rgb = (rgb + prev[..., :3].astype(np.float32) / 255.0 * sample_index) / float(sample_index + 1)
    q = np.clip((rgb.astype(np.float32) * 256.0).astype(np.int64), 0, 255).astype(np.uint8)
    out = np.full(results.shape[:2] + (4,), 255, np.uint8)
    out[..., :3] = q
    return out


def psnr(a: np.ndarray, b: np.ndarray, peak: float = 1.0) -> float:
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * math.log10(peak * peak / mse)
