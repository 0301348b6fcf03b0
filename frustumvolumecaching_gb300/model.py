"""Seeded synthetic NeRF models written in the reference's nerfacc export format.

The reference loads a model directory holding ``config.json`` plus fp16 blobs
``pos_enc.dat``, ``mlp_base.dat``, ``mlp_head.dat`` and a uint8
``occupancy_grid.dat`` (src/loader.cu:232-285, include/parse_helper.h:25-63).
No trained model ships with the reference, so workloads are generated here from
a seed: hash tables uniform in +-1e-2, Xavier-uniform MLP weights, and an
occupancy grid obtained by thresholding the network's density at cell centres.

Parameter layout (what the loader and the kernels read):

* ``pos_enc.dat``: the hash tables of all levels back to back; level ``l`` has
  ``hashmap_size(l)`` entries of ``F`` fp16 features (entry-major).
* ``mlp_base.dat`` / ``mlp_head.dat``: each layer's weight matrix row-major as
  ``[n_out_padded x n_in_padded]`` fp16, layers in order, no biases (tcnn's
  FullyFusedMLP has none; include/nerf_network.h:92-118).
* ``occupancy_grid.dat``: one byte per cell, ``l*R^3 + x*R^2 + y*R + z``
  (src/loader.cu:20-38 reads it in that order).

Extension keys in ``config.json`` (absent from nerfacc exports, defaulted to the
reference behaviour by the loader): ``mlp_head.n_latents`` and
``mlp_head.first_latent_is_density`` select which density-network outputs feed
the color head (NerfNetwork::latent_offset, include/nerf_network.h:334-337).
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

GRID_RES = 128  # DEFAULT_GRID_RESOLUTION, include/renderer_common.h:10

# Real spherical harmonics up to degree 4 (l = 0..3, 16 values) on a unit
# direction, following Sloan, "Stupid Spherical Harmonics Tricks", appendix A1;
# the same sign convention as src/my_fully_fused_mlp.cu:216-233.
_SQ = math.sqrt
_PI = math.pi
SH_C = {
    "c0": 1.0 / (2.0 * _SQ(_PI)),
    "c1": _SQ(3.0) / (2.0 * _SQ(_PI)),
    "c2a": _SQ(15.0) / (2.0 * _SQ(_PI)),
    "c2b": _SQ(5.0) / (4.0 * _SQ(_PI)),
    "c2c": _SQ(15.0) / (4.0 * _SQ(_PI)),
    "c3a": _SQ(70.0) / (8.0 * _SQ(_PI)),
    "c3b": _SQ(105.0) / (2.0 * _SQ(_PI)),
    "c3c": _SQ(42.0) / (8.0 * _SQ(_PI)),
    "c3d": _SQ(7.0) / (4.0 * _SQ(_PI)),
    "c3e": _SQ(105.0) / (4.0 * _SQ(_PI)),
}


def sh4(d: np.ndarray) -> np.ndarray:
    """16 SH values of directions ``d`` ([N,3], components in [-1,1])."""
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xy, xz, yz, x2, y2, z2 = x * y, x * z, y * z, x * x, y * y, z * z
    c = SH_C
    out = np.stack([
        np.full_like(x, c["c0"]),
        -c["c1"] * y, c["c1"] * z, -c["c1"] * x,
        c["c2a"] * xy, -c["c2a"] * yz, c["c2b"] * (3.0 * z2 - 1.0), -c["c2a"] * xz,
        c["c2c"] * (x2 - y2),
        c["c3a"] * y * (-3.0 * x2 + y2), c["c3b"] * xy * z, c["c3c"] * y * (1.0 - 5.0 * z2),
        c["c3d"] * z * (5.0 * z2 - 3.0), c["c3c"] * x * (1.0 - 5.0 * z2),
        c["c3e"] * z * (x2 - y2), c["c3a"] * x * (-x2 + 3.0 * y2),
    ], axis=1)
    return out


@dataclass
class HashLevel:
    scale: float      # float32 value used on the device
    res: int          # ceil(scale) + 1
    size: int         # entries in the level's table
    offset: int       # first entry of the level
    dense: bool       # res^3 <= size: direct indexing instead of hashing


def hash_grid_levels(n_levels: int, base_res: int, per_level_scale: float, log2_T: int,
                     scales: list | None = None) -> list[HashLevel]:
    """Per-level layout of the multiresolution hash grid.

    Multiresolution levels with geometric growth (Mueller et al. 2022,
    "Instant Neural Graphics Primitives", sec. 3): ``scale_l = N_min*b^l - 1``
    in float32 (the +1 vertex per axis gives ``res_l = ceil(scale_l) + 1``);
    a level keeps ``min(round_up(res^3, 8), T)`` entries and is indexed densely
    when the grid fits, else by the spatial hash.  The loader computes the
    same layout in C++ and checks the table size against ``pos_enc.dat``.
    """
    f32 = np.float32
    log2_b = np.log2(f32(per_level_scale), dtype=f32)
    T = 1 << log2_T
    levels = []
    off = 0
    for l in range(n_levels):
        scale = f32(np.exp2(f32(l) * log2_b, dtype=f32) * f32(base_res) - f32(1.0))
        if scales is not None:  # explicit per-level scales (config.json fvc_level_scales)
            scale = f32(scales[l])
        res = int(math.ceil(float(scale))) + 1
        n = res ** 3
        n = (n + 7) // 8 * 8
        size = min(n, T)
        levels.append(HashLevel(float(scale), res, size, off, res ** 3 <= size))
        off += size
    return levels


def hash_encode(pos: np.ndarray, table: np.ndarray, levels: list[HashLevel], F: int = 2) -> np.ndarray:
    """Hash-grid features of contracted positions ``pos`` ([N,3] in [0,1]).

    Per level: ``p = scale*x + 0.5``, corner = floor(p), trilinear weights
    from the fraction; dense index ``x + y*res + z*res^2`` or the hash
    ``x*1 ^ y*2654435761 ^ z*805459861`` (uint32), both modulo the level size.
    Accumulates in float64; ``table`` is [entries, F] float (fp16 values)."""
    N = pos.shape[0]
    out = np.zeros((N, len(levels) * F), dtype=np.float64)
    p32 = pos.astype(np.float32)
    for li, lv in enumerate(levels):
        # fmaf(scale, x, 0.5): the float32 product is exact in float64, one rounding after the add
        p = (np.float64(np.float32(lv.scale)) * p32.astype(np.float64) + 0.5).astype(np.float32)
        g = np.floor(p)
        fr = (p - g).astype(np.float64)
        gi = g.astype(np.int64).astype(np.uint32)
        acc = np.zeros((N, F), dtype=np.float64)
        for c in range(8):
            bx, by, bz = (c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1
            cx = gi[:, 0] + np.uint32(bx)
            cy = gi[:, 1] + np.uint32(by)
            cz = gi[:, 2] + np.uint32(bz)
            w = (fr[:, 0] if bx else 1 - fr[:, 0]) * (fr[:, 1] if by else 1 - fr[:, 1]) * (fr[:, 2] if bz else 1 - fr[:, 2])
            if lv.dense:
                idx = (cx.astype(np.uint64) + cy.astype(np.uint64) * lv.res + cz.astype(np.uint64) * lv.res * lv.res)
            else:
                h = (cx * np.uint32(1)) ^ (cy * np.uint32(2654435761)) ^ (cz * np.uint32(805459861))
                idx = h.astype(np.uint64)
            idx = (idx % np.uint64(lv.size)).astype(np.int64) + lv.offset
            acc += w[:, None] * table[idx]
        out[:, li * F:(li + 1) * F] = acc
    return out


def contract(world: np.ndarray, scene: dict) -> np.ndarray:
    """apply_contraction (include/raymarch_common.h:610-653), float64."""
    if scene["contraction"] == "linf":
        f = np.asarray(scene["contraction_aabb"][:3], np.float64)
        t = np.asarray(scene["contraction_aabb"][3:], np.float64)
        u = (world - f) / (t - f) * 2.0 - 1.0
        n = np.max(np.abs(u), axis=1, keepdims=True)
        fac = np.maximum(n, 1.0)
        c = (2.0 - 1.0 / fac) * (u / fac)
        return c / 4.0 + 0.5
    f = np.asarray(scene["aabb"][:3], np.float64)
    t = np.asarray(scene["aabb"][3:], np.float64)
    return (world - f) / (t - f)


@dataclass
class ModelSpec:
    """One seeded synthetic workload."""
    name: str
    seed: int
    aabb: list
    grid_nlvl: int = 1
    contraction: str = "aabb"          # "aabb" or "linf"
    contraction_aabb: list = field(default_factory=lambda: [-1.5, -1.5, -1.5, 1.5, 1.5, 1.5])
    cone_angle: float = 0.0
    stepsize: float = 3.0 / 1024.0
    near: float = 0.0
    far: float = 1e10
    alpha_thre: float = 0.0
    n_levels: int = 16
    F: int = 2
    log2_T: int = 16
    base_res: int = 16
    per_level_scale: float = 1.447
    width: int = 64
    n_latents: int = 8
    first_latent_is_density: bool = False
    head_hidden_layers: int = 2
    table_range: float = 1e-2
    occupancy_fraction: float = 0.12
    occupancy_cascades: str = "all"     # "all": threshold every cascade; "inner": outer cascades empty
    view_dependent: bool = False        # split head (mlp_first_head): latents from a first head on an initial direction
    freq_encoding_degree: int = 0       # 4: the head also reads sin / cos(pi 2^k p) of the contracted position, k < 4


def spec_config1() -> ModelSpec:
    """Plain 256x256 workload: 1 cascade over [-1.5,1.5]^3, 2^16 entries/level."""
    return ModelSpec(name="c1_plain256", seed=1001, aabb=[-1.5, -1.5, -1.5, 1.5, 1.5, 1.5])


def spec_config2() -> ModelSpec:
    """Cached 1080p workload: 3 cascades over [-6,6]^3 with the L-infinity
    scene contraction around [-1.5,1.5]^3, 2^19 entries/level; step
    parameters are the reference loader defaults cone 1/256, step sqrt(3)/1024
    (src/loader.cu:190-191)."""
    return ModelSpec(name="c2_cached1080", seed=1002, aabb=[-6.0, -6.0, -6.0, 6.0, 6.0, 6.0], grid_nlvl=3,
                     contraction="linf", cone_angle=1.0 / 256.0, stepsize=math.sqrt(3.0) / 1024.0, log2_T=19)


def spec_config5(target: bool = False) -> ModelSpec:
    """Differentiable-render workload: the config-1 architecture and scene box
    with 2^19 entries/level; the target image comes from a second network of
    the same architecture seeded differently."""
    return ModelSpec(name="c5_target" if target else "c5_train", seed=1105 if target else 1005,
                     aabb=[-1.5, -1.5, -1.5, 1.5, 1.5, 1.5], log2_T=19)


def spec_tiny(seed: int = 7, nlvl: int = 1, cone: float = 0.0, log2_T: int = 12) -> ModelSpec:
    """Small model for fast CPU tests (tables 2^12, 16 levels)."""
    if nlvl == 1:
        return ModelSpec(name=f"tiny{seed}", seed=seed, aabb=[-1.5, -1.5, -1.5, 1.5, 1.5, 1.5], cone_angle=cone, log2_T=log2_T)
    return ModelSpec(name=f"tiny{seed}_c{nlvl}", seed=seed, aabb=[-6.0, -6.0, -6.0, 6.0, 6.0, 6.0], grid_nlvl=nlvl,
                     contraction="linf", cone_angle=cone if cone > 0 else 1.0 / 256.0,
                     stepsize=math.sqrt(3.0) / 1024.0, log2_T=log2_T)


def _xavier(rng, n_out, n_in, n_out_pad, n_in_pad):
    lim = math.sqrt(6.0 / (n_in + n_out))
    w = np.zeros((n_out_pad, n_in_pad), np.float32)
    w[:n_out, :n_in_pad] = rng.uniform(-lim, lim, size=(n_out, n_in_pad))
    return w.astype(np.float16)


def _pad16(n):
    return (n + 15) // 16 * 16


class SyntheticModel:
    """Parameters of a generated model held in numpy (fp16 values)."""

    def __init__(self, spec: ModelSpec):
        self.spec = spec
        rng = np.random.default_rng([spec.seed, 0])
        self.levels = hash_grid_levels(spec.n_levels, spec.base_res, spec.per_level_scale, spec.log2_T)
        n_entries = self.levels[-1].offset + self.levels[-1].size
        self.table = rng.uniform(-spec.table_range, spec.table_range, size=(n_entries, spec.F)).astype(np.float16)
        enc_w = spec.n_levels * spec.F
        n_out = 1 + spec.n_latents if not spec.first_latent_is_density else spec.n_latents
        self.n_base_out = n_out
        self.base = [_xavier(rng, spec.width, enc_w, spec.width, _pad16(enc_w)),
                     _xavier(rng, n_out, spec.width, _pad16(n_out), spec.width)]
        # the head reads [latents | SH of the direction (16)], a view-dependent head also the SH
        # difference to the initial direction (16), and with a frequency encoding the 6 * degree
        # sines and cosines of the position (include/nerf_network.h:55-81,204-257)
        head_in = spec.n_latents + (32 if spec.view_dependent else 16) + 6 * spec.freq_encoding_degree
        self.head_in = head_in
        head_in_pad = _pad16(head_in)
        hl = [_xavier(rng, spec.width, head_in, spec.width, head_in_pad)]
        for _ in range(spec.head_hidden_layers - 1):
            hl.append(_xavier(rng, spec.width, spec.width, spec.width, spec.width))
        hl.append(_xavier(rng, 3, spec.width, 16, spec.width))
        self.head = hl
        # the first head: [density outputs (16) | SH of the initial direction (16)] -> 64 -> n_latents
        self.first = ([_xavier(rng, spec.width, 32, spec.width, 32), _xavier(rng, spec.n_latents, spec.width, 16, spec.width)]
                      if spec.view_dependent else None)
        self.occupancy = None

    # -- evaluation (float64 with fp16 rounding of layer outputs like tcnn) --
    def base_outputs(self, pos: np.ndarray) -> np.ndarray:
        feat = hash_encode(pos, self.table.astype(np.float64), self.levels, self.spec.F)
        x = feat.astype(np.float16).astype(np.float64)
        W0 = self.base[0].astype(np.float64)
        W1 = self.base[1].astype(np.float64)
        h = np.maximum(x @ W0[:, :x.shape[1]].T, 0.0).astype(np.float16).astype(np.float64)
        return (h @ W1.T).astype(np.float16).astype(np.float64)

    def log_density(self, pos: np.ndarray, chunk: int = 1 << 18) -> np.ndarray:
        out = np.empty(pos.shape[0], np.float64)
        for s in range(0, pos.shape[0], chunk):
            out[s:s + chunk] = self.base_outputs(pos[s:s + chunk])[:, 0 if not self.spec.first_latent_is_density else 0]
        return out

    def scene_dict(self) -> dict:
        s = self.spec
        return {"aabb": s.aabb, "contraction": s.contraction, "contraction_aabb": s.contraction_aabb}

    def cell_centres_world(self, level: int) -> np.ndarray:
        """World positions of all cell centres of one cascade, in file order
        (x-major: x*R^2 + y*R + z), inverse of world_to_aabb_unit and the
        cascade scaling of grid_occupied_at (include/raymarch_common.h:660-693)."""
        s = self.spec
        R = GRID_RES
        i = (np.arange(R, dtype=np.float64) + 0.5) / R
        X, Y, Z = np.meshgrid(i, i, i, indexing="ij")
        pum = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        u = (pum - 0.5) * (2.0 ** level) + 0.5
        sc = 2.0 ** (s.grid_nlvl - 1)
        f = np.asarray(s.aabb[:3], np.float64)
        t = np.asarray(s.aabb[3:], np.float64)
        return u * ((t - f) / sc) + f / sc

    def build_occupancy(self) -> np.ndarray:
        s = self.spec
        R3 = GRID_RES ** 3
        occ = np.zeros(R3 * s.grid_nlvl, np.uint8)
        for l in range(s.grid_nlvl):
            if s.occupancy_cascades == "inner" and l > 0:
                continue
            world = self.cell_centres_world(l)
            ld = self.log_density(contract(world, self.scene_dict()))
            thr = np.quantile(ld, 1.0 - s.occupancy_fraction)
            occ[l * R3:(l + 1) * R3] = (ld > thr).astype(np.uint8)
        self.occupancy = occ
        return occ

    # -- export ---------------------------------------------------------------
    def config_json(self) -> dict:
        s = self.spec
        scene = {
            "grid_resolution": GRID_RES, "grid_nlvl": s.grid_nlvl, "aabb": s.aabb,
            "is_open_gl": False, "alpha_thre": s.alpha_thre, "cone_angle": s.cone_angle,
            "stepsize": s.stepsize, "near": s.near, "far": s.far,
        }
        if s.contraction == "linf":
            scene["contraction"] = {"type": "AABB_LINF", "aabb": s.contraction_aabb}
        enc = {"otype": "HashGrid", "n_levels": s.n_levels, "n_features_per_level": s.F,
               "log2_hashmap_size": s.log2_T, "base_resolution": s.base_res, "per_level_scale": s.per_level_scale,
               "fvc_level_scales": [float(lv.scale) for lv in self.levels]}
        net = {"otype": "FullyFusedMLP", "activation": "ReLU", "output_activation": "None",
               "n_neurons": s.width, "n_hidden_layers": 1}
        head_net = dict(net, n_hidden_layers=s.head_hidden_layers)
        sh_enc = {"otype": "Composite", "nested": [{"otype": "SphericalHarmonics", "degree": 4, "n_dims_to_encode": 3}]}
        out = {
            "scene": scene,
            "mlp_base": {"encoding": enc, "network": net, "n_output": self.n_base_out},
            "mlp_head": {"encoding": sh_enc,
                "network": head_net, "n_input": self.head_in, "n_latents": s.n_latents,
                "first_latent_is_density": s.first_latent_is_density,
                "freq_encoding_degree": s.freq_encoding_degree},
            "synthetic": {"seed": s.seed, "name": s.name, "occupancy_fraction": s.occupancy_fraction,
                          "table_range": s.table_range,
                          "hashmap_sizes": [lv.size for lv in self.levels]},
        }
        if s.view_dependent:  # loaded by NerfNetwork::init_viewdep (src/loader.cu:251-262)
            out["mlp_first_head"] = {"encoding": sh_enc, "network": dict(net), "n_input": 32, "n_output": s.n_latents,
                                     "first_latent_is_density": s.first_latent_is_density}
        return out

    def write(self, out_dir: str) -> str:
        os.makedirs(out_dir, exist_ok=True)
        if self.occupancy is None:
            self.build_occupancy()
        with open(os.path.join(out_dir, "config.json"), "w") as f:
            json.dump(self.config_json(), f, indent=1)
        self.table.tofile(os.path.join(out_dir, "pos_enc.dat"))
        np.concatenate([w.ravel() for w in self.base]).tofile(os.path.join(out_dir, "mlp_base.dat"))
        np.concatenate([w.ravel() for w in self.head]).tofile(os.path.join(out_dir, "mlp_head.dat"))
        if self.first is not None:
            np.concatenate([w.ravel() for w in self.first]).tofile(os.path.join(out_dir, "mlp_first_head.dat"))
        self.occupancy.tofile(os.path.join(out_dir, "occupancy_grid.dat"))
        return out_dir


def default_model_root() -> str:
    return os.environ.get("FVC_MODEL_DIR", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "_models"))


def model_dir_name(spec: ModelSpec) -> str:
    vd = "_vd" if spec.view_dependent else ""
    fq = f"_freq{spec.freq_encoding_degree}" if spec.freq_encoding_degree else ""
    return (f"{spec.name}_s{spec.seed}_T{spec.log2_T}_n{spec.grid_nlvl}_o{int(round(spec.occupancy_fraction * 1000))}"
            f"{spec.occupancy_cascades}{vd}{fq}")


def ensure_model(spec: ModelSpec, root: str | None = None) -> str:
    """Generate (once) and return the export directory of ``spec``."""
    root = root or default_model_root()
    d = os.path.join(root, model_dir_name(spec))
    if not os.path.exists(os.path.join(d, "occupancy_grid.dat")):
        tmp = f"{d}.tmp{os.getpid()}"
        SyntheticModel(spec).write(tmp)
        try:
            os.rename(tmp, d)
        except OSError:
            import shutil
            shutil.rmtree(tmp, ignore_errors=True)
    return d
