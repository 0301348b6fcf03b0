"""Oracle restatement of the reference's instant-ngp snapshot loader.

TEST INFRASTRUCTURE: only tests may use this module, as the checker of the
library's .ingp reader (never as the thing measured or shipped).

It follows load_ingp_snapshot (src/loader.cu:146-230) and
ingp_density_grid_to_occupancy_grid (src/loader.cu:73-114) and writes the
result as a nerfacc export directory (config.json + four blobs) that
``oracle.OracleModel`` loads:
- the document: a msgpack map, deflate-compressed with a gzip or zlib wrapper
  or stored without one (the reference reads it through zstr, which detects
  the wrapper); decompression here is Python's zlib, the msgpack decoder is
  written below from the msgpack specification;
- scene: 128^3 grid, log2(aabb_scale)+1 cascades, normalized, the snapshot's
  aabb with AABB contraction, alpha threshold 0, cone 1/256 for more than one
  cascade (else 0), step sqrt(3)/1024, near 0, far 1e10 (:176-195);
- hash grid: the snapshot's encoding with per_level_scale =
  exp(log(2048 aabb_scale / base_resolution) / (n_levels - 1)) in float32
  (:197-202; libm's expf/logf where available, as the C++ float overloads);
- density MLP with 16 outputs, color MLP from rgb_network with the
  dir_encoding SH degree (:203-208); the parameter blob split in the order of
  NerfNetwork::set_params (include/nerf_network.h:284-298): density MLP
  [64 x 32][16 x 64], color MLP [64 x 32]([64 x 64]...)[16 x 64], hash grid;
- occupancy: density grid fp16, Morton order per cascade, occupied where the
  density exceeds min(0.01, mean over the first cascade of max(d, 0)),
  written as the linear uchar grid [cascade][x][y][z].
"""
import ctypes
import ctypes.util
import json
import math
import os
import struct
import zlib

import numpy as np

GRID_RES = 128


class MsgpackError(ValueError):
    pass


def _decode(buf: bytes, pos: int):
    """One msgpack value at ``pos``: (value, next position)."""
    if pos >= len(buf):
        raise MsgpackError("truncated document")
    c = buf[pos]
    pos += 1

    def take(n):
        nonlocal pos
        if pos + n > len(buf):
            raise MsgpackError("truncated document")
        v = buf[pos:pos + n]
        pos += n
        return v

    def uint(n):
        return int.from_bytes(take(n), "big")

    def seq(n):
        nonlocal pos
        out = []
        for _ in range(n):
            v, pos = _decode(buf, pos)
            out.append(v)
        return out

    def mapping(n):
        nonlocal pos
        out = {}
        for _ in range(n):
            k, pos = _decode(buf, pos)
            v, pos = _decode(buf, pos)
            out[k] = v
        return out

    if c <= 0x7F:
        return c, pos
    if c >= 0xE0:
        return c - 256, pos
    if 0x80 <= c <= 0x8F:
        return mapping(c & 0x0F), pos
    if 0x90 <= c <= 0x9F:
        return seq(c & 0x0F), pos
    if 0xA0 <= c <= 0xBF:
        return take(c & 0x1F).decode(), pos
    if c == 0xC0:
        return None, pos
    if c in (0xC2, 0xC3):
        return c == 0xC3, pos
    if c in (0xC4, 0xC5, 0xC6):
        return bytes(take(uint({0xC4: 1, 0xC5: 2, 0xC6: 4}[c]))), pos
    if c == 0xCA:
        return struct.unpack(">f", take(4))[0], pos
    if c == 0xCB:
        return struct.unpack(">d", take(8))[0], pos
    if c in (0xCC, 0xCD, 0xCE, 0xCF):
        return uint({0xCC: 1, 0xCD: 2, 0xCE: 4, 0xCF: 8}[c]), pos
    if c in (0xD0, 0xD1, 0xD2, 0xD3):
        n = {0xD0: 1, 0xD1: 2, 0xD2: 4, 0xD3: 8}[c]
        return int.from_bytes(take(n), "big", signed=True), pos
    if c in (0xD9, 0xDA, 0xDB):
        return take(uint({0xD9: 1, 0xDA: 2, 0xDB: 4}[c])).decode(), pos
    if c in (0xDC, 0xDD):
        return seq(uint(2 if c == 0xDC else 4)), pos
    if c in (0xDE, 0xDF):
        return mapping(uint(2 if c == 0xDE else 4)), pos
    raise MsgpackError(f"unsupported msgpack type byte 0x{c:02x}")


def unpack(buf: bytes):
    v, _ = _decode(buf, 0)
    return v


def decompress(data: bytes) -> bytes:
    if data[:2] == b"\x1f\x8b":
        return zlib.decompress(data, 16 + zlib.MAX_WBITS)
    if len(data) >= 2 and (data[0] & 0x0F) == 8 and (data[0] >> 4) <= 7 and ((data[0] << 8) | data[1]) % 31 == 0:
        return zlib.decompress(data)
    return data


def _float_fns():
    name = ctypes.util.find_library("m")
    try:
        m = ctypes.CDLL(name or "libm.so.6")
        expf, logf = m.expf, m.logf
        for f in (expf, logf):
            f.restype = ctypes.c_float
            f.argtypes = [ctypes.c_float]
        return expf, logf
    except (OSError, AttributeError):
        return (lambda x: float(np.float32(math.exp(x)))), (lambda x: float(np.float32(math.log(x))))


def per_level_scale(aabb_scale: int, base_res: int, n_levels: int) -> float:
    expf, logf = _float_fns()
    f32 = np.float32
    arg = f32(f32(2048.0) * f32(aabb_scale)) / f32(base_res)
    return float(f32(expf(float(f32(f32(logf(float(arg))) / f32(n_levels - 1))))))


def _compact(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint32) & np.uint32(0x49249249)
    v = (v | (v >> 2)) & np.uint32(0xC30C30C3)
    v = (v | (v >> 4)) & np.uint32(0x0F00F00F)
    v = (v | (v >> 8)) & np.uint32(0xFF0000FF)
    v = (v | (v >> 16)) & np.uint32(0x0000FFFF)
    return v


def occupancy_from_density(density: np.ndarray, nlvl: int) -> np.ndarray:
    """ingp_density_grid_to_occupancy_grid (src/loader.cu:73-114): fp16 density
    [cascade][Morton index] -> linear uchar occupancy [cascade][x][y][z]."""
    vals = GRID_RES ** 3
    d = density.astype(np.float32).reshape(nlvl, vals)
    mean = float(np.sum(np.maximum(d[0], 0.0).astype(np.float64) / vals))
    thresh = min(np.float32(0.01), np.float32(mean))
    i = np.arange(vals, dtype=np.uint32)
    lin = _compact(i).astype(np.int64) * GRID_RES * GRID_RES + _compact(i >> 1).astype(np.int64) * GRID_RES + \
        _compact(i >> 2).astype(np.int64)
    occ = np.zeros((nlvl, vals), np.uint8)
    for lv in range(nlvl):
        occ[lv, lin] = (d[lv] > thresh).astype(np.uint8)
    return occ.reshape(-1)


def snapshot_to_export(snapshot: str, out_dir: str) -> dict:
    """Writes the nerfacc export equivalent of an .ingp snapshot; returns its config."""
    with open(snapshot, "rb") as f:
        doc = unpack(decompress(f.read()))
    if not isinstance(doc, dict) or "snapshot" not in doc:
        raise ValueError("no snapshot")
    snap = doc["snapshot"]
    if snap.get("mode") != "nerf":
        raise ValueError("not a nerf snapshot")
    aabb_scale = int(snap["nerf"]["aabb_scale"])
    nlvl = int(round(math.log2(aabb_scale))) + 1
    amin, amax = snap["aabb"]["min"], snap["aabb"]["max"]
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    enc = doc["encoding"]
    n_levels = int(enc.get("n_levels", 16))
    base_res = int(enc.get("base_resolution", 16))
    rgb = doc["rgb_network"]
    head_hidden = int(rgb.get("n_hidden_layers", 2))
    sh = 4
    nested = doc.get("dir_encoding", {}).get("nested")
    if nested:
        sh = int(nested[0].get("degree", 4))
    cfg = {
        "scene": {"grid_resolution": GRID_RES, "grid_nlvl": nlvl, "normalized": True,
                  "aabb": [f32(v) for v in amin] + [f32(v) for v in amax], "is_open_gl": False, "alpha_thre": 0.0,
                  "cone_angle": 0.0 if nlvl <= 1 else f32(1.0 / 256.0), "stepsize": f32(np.sqrt(np.float32(3.0)) / np.float32(1024.0)),
                  "near": 0.0, "far": f32(1e10)},
        "mlp_base": {"encoding": {"n_levels": n_levels, "n_features_per_level": int(enc.get("n_features_per_level", 2)),
                                  "log2_hashmap_size": int(enc.get("log2_hashmap_size", 19)), "base_resolution": base_res,
                                  "per_level_scale": per_level_scale(aabb_scale, base_res, n_levels)},
                     "network": {"n_neurons": int(doc["network"].get("n_neurons", 64)),
                                 "n_hidden_layers": int(doc["network"].get("n_hidden_layers", 1))},
                     "n_output": 16},
        "mlp_head": {"network": {"n_neurons": int(rgb.get("n_neurons", 64)), "n_hidden_layers": head_hidden},
                     "encoding": {"nested": [{"degree": sh}]}, "first_latent_is_density": True, "n_latents": 16,
                     "n_input": 32},
    }
    params = np.frombuffer(snap["params_binary"], np.uint16)
    n_base = 64 * 32 + 16 * 64
    n_head = 64 * 32 + max(0, head_hidden - 1) * 64 * 64 + 16 * 64
    density = np.frombuffer(snap["density_grid_binary"], np.float16)
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "config.json"), "w") as f:
        json.dump(cfg, f)
    params[:n_base].tofile(os.path.join(out_dir, "mlp_base.dat"))
    params[n_base:n_base + n_head].tofile(os.path.join(out_dir, "mlp_head.dat"))
    params[n_base + n_head:].tofile(os.path.join(out_dir, "pos_enc.dat"))
    occupancy_from_density(density, nlvl).tofile(os.path.join(out_dir, "occupancy_grid.dat"))
    return cfg
