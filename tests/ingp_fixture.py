"""Synthetic instant-ngp snapshots (.ingp) for the loader tests.

A snapshot is the msgpack document the reference's loader reads
(src/loader.cu:146-230): ``snapshot.{mode, nerf.aabb_scale, aabb.{min,max},
params_binary, density_grid_binary}`` and the root ``encoding``, ``network``,
``dir_encoding`` and ``rgb_network`` configurations.  The msgpack encoder below
is written from the msgpack specification; the document is wrapped with
Python's gzip / zlib (or left uncompressed).
"""
import gzip
import math
import struct
import zlib

import numpy as np

from frustumvolumecaching_gb300 import model as fmodel

GRID_RES = 128


def pack(v) -> bytes:
    if v is None:
        return b"\xc0"
    if v is True:
        return b"\xc3"
    if v is False:
        return b"\xc2"
    if isinstance(v, int):
        if 0 <= v <= 0x7F:
            return bytes([v])
        if -32 <= v < 0:
            return bytes([v & 0xFF])
        if 0 <= v <= 0xFFFF:
            return b"\xcd" + struct.pack(">H", v)
        if 0 <= v <= 0xFFFFFFFF:
            return b"\xce" + struct.pack(">I", v)
        return b"\xd3" + struct.pack(">q", v)
    if isinstance(v, float):
        if float(np.float32(v)) == v:
            return b"\xca" + struct.pack(">f", v)
        return b"\xcb" + struct.pack(">d", v)
    if isinstance(v, str):
        b = v.encode()
        if len(b) < 32:
            return bytes([0xA0 | len(b)]) + b
        return b"\xd9" + bytes([len(b)]) + b if len(b) < 256 else b"\xda" + struct.pack(">H", len(b)) + b
    if isinstance(v, (bytes, bytearray)):
        n = len(v)
        if n < 256:
            return b"\xc4" + bytes([n]) + bytes(v)
        if n < 65536:
            return b"\xc5" + struct.pack(">H", n) + bytes(v)
        return b"\xc6" + struct.pack(">I", n) + bytes(v)
    if isinstance(v, (list, tuple)):
        head = bytes([0x90 | len(v)]) if len(v) < 16 else b"\xdc" + struct.pack(">H", len(v))
        return head + b"".join(pack(x) for x in v)
    if isinstance(v, dict):
        head = bytes([0x80 | len(v)]) if len(v) < 16 else b"\xde" + struct.pack(">H", len(v))
        return head + b"".join(pack(k) + pack(x) for k, x in v.items())
    raise TypeError(type(v))


def _expand(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint32) & np.uint32(0x3FF)
    v = (v | (v << 16)) & np.uint32(0x030000FF)
    v = (v | (v << 8)) & np.uint32(0x0300F00F)
    v = (v | (v << 4)) & np.uint32(0x030C30C3)
    v = (v | (v << 2)) & np.uint32(0x09249249)
    return v


def morton_from_linear() -> np.ndarray:
    """The Morton index of each linear cell (x*R^2 + y*R + z) of one cascade."""
    n = GRID_RES ** 3
    i = np.arange(n, dtype=np.int64)
    x, y, z = i // (GRID_RES * GRID_RES), (i // GRID_RES) % GRID_RES, i % GRID_RES
    return (_expand(x) | (_expand(y) << 1) | (_expand(z) << 2)).astype(np.int64)


def ingp_model(seed: int = 31, aabb_scale: int = 2):
    """An instant-ngp-shaped synthetic model: 16-level, 2-feature hash grid
    (2^12 entries per level), density MLP 32-64-16 whose first output is the
    density, color MLP (16 latents + 16 SH)-64-64-3 (fp16 blobs), and a linear
    occupancy grid: a ball of radius 0.35 around each cascade's centre plus
    5 % scattered cells."""
    nlvl = int(round(math.log2(aabb_scale))) + 1
    spec = fmodel.ModelSpec(name=f"ingp_like{seed}_s{aabb_scale}", seed=seed, aabb=[0.0] * 3 + [1.0] * 3,
                            grid_nlvl=nlvl, n_latents=16, first_latent_is_density=True, log2_T=12,
                            per_level_scale=float((2048.0 * aabb_scale / 16.0) ** (1.0 / 15.0)))
    m = fmodel.SyntheticModel(spec)
    wb = np.concatenate([w.ravel() for w in m.base]).view(np.uint16)
    wh = np.concatenate([w.ravel() for w in m.head]).view(np.uint16)
    tab = m.table.ravel().view(np.uint16)
    rng = np.random.default_rng([seed, 7])
    c = (np.arange(GRID_RES) + 0.5) / GRID_RES - 0.5
    r2 = c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2
    ball = (r2 < 0.35 ** 2).ravel()
    occ = np.concatenate([(ball | (rng.random(GRID_RES ** 3) < 0.05)).astype(np.uint8) for _ in range(nlvl)])
    return spec, wb, wh, tab, occ


def density_grid(occ_linear: np.ndarray, nlvl: int, seed: int, low: bool = False) -> np.ndarray:
    """fp16 density grid in Morton order per cascade: occupied cells get
    densities well above 0.01, free cells values at or below it (negative
    ones too); ``low`` scales everything down so that the first cascade's mean
    density falls below 0.01 and becomes the threshold."""
    rng = np.random.default_rng(seed)
    n = GRID_RES ** 3
    mort = morton_from_linear()
    out = np.zeros((nlvl, n), np.float16)
    for lv in range(nlvl):
        occ = occ_linear.reshape(nlvl, n)[lv].astype(bool)
        dens = np.where(occ, rng.uniform(0.05, 4.0, n), rng.uniform(-0.5, 0.0099, n))
        if low:
            dens = np.where(occ, rng.uniform(0.0, 0.05, n), rng.uniform(-0.01, 0.0005, n))
        out[lv, mort] = dens.astype(np.float16)
    return out.reshape(-1)


def write_snapshot(path, aabb_scale: int, params: np.ndarray, density: np.ndarray, wrapper: str = "gzip",
                   mode: str = "nerf", head_hidden: int = 2, n_levels: int = 16, n_features: int = 2,
                   log2_T: int = 12, drop=()) -> str:
    lo, hi = 0.5 - aabb_scale / 2.0, 0.5 + aabb_scale / 2.0
    snap = {"mode": mode, "nerf": {"aabb_scale": aabb_scale, "rgb": {"measured_cam_focal_length": 1.0}},
            "aabb": {"min": [lo] * 3, "max": [hi] * 3},
            "params_binary": params.astype(np.uint16).tobytes(), "density_grid_binary": density.astype(np.float16).tobytes(),
            "density_grid_size": GRID_RES, "version": 1}
    doc = {"encoding": {"otype": "HashGrid", "n_levels": n_levels, "n_features_per_level": n_features,
                        "log2_hashmap_size": log2_T, "base_resolution": 16},
           "network": {"otype": "FullyFusedMLP", "activation": "ReLU", "output_activation": "None", "n_neurons": 64,
                       "n_hidden_layers": 1},
           "dir_encoding": {"otype": "Composite",
                            "nested": [{"n_dims_to_encode": 3, "otype": "SphericalHarmonics", "degree": 4},
                                       {"otype": "Identity", "n_bins": 4, "degree": 4}]},
           "rgb_network": {"otype": "FullyFusedMLP", "activation": "ReLU", "output_activation": "None", "n_neurons": 64,
                           "n_hidden_layers": head_hidden},
           "snapshot": snap}
    for k in drop:
        (snap if k in snap else doc).pop(k)
    raw = pack(doc)
    if wrapper == "gzip":
        data = gzip.compress(raw)
    elif wrapper == "zlib":
        data = zlib.compress(raw, 6)
    elif wrapper == "stored":
        data = zlib.compress(raw, 0)
    elif wrapper == "fixed":
        c = zlib.compressobj(6, zlib.DEFLATED, zlib.MAX_WBITS, 8, zlib.Z_FIXED)
        data = c.compress(raw) + c.flush()
    else:
        data = raw
    with open(path, "wb") as f:
        f.write(data)
    return str(path)


def make_snapshot(tmp_path, name="scene.ingp", seed=31, aabb_scale=2, wrapper="gzip", low=False, **kw) -> str:
    spec, wb, wh, tab, occ = ingp_model(seed, aabb_scale)
    dens = density_grid(occ, spec.grid_nlvl, seed + 1, low=low)
    return write_snapshot(tmp_path / name, aabb_scale, np.concatenate([wb, wh, tab]), dens, wrapper=wrapper, **kw)
