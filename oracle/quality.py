"""Image quality of the GPU renders against the float64 oracle.

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's untimed quality
rows as the checker.  The product package never imports it.

The metric's quality clause ("cached at dPSNR <= 0.1 dB vs the FP64 oracle")
is measured on the final white-background pixel colour (rgb + T, the value
writeImageBuffer_performance_kernel quantises, src/performance_renderer.cu:
127-149) of a band of image rows:

    psnr_plain_db         GPU plain render       vs FP64 plain oracle
    psnr_cached_db        GPU cached render      vs FP64 plain oracle
    psnr_cached_fp64_db   FP64 cached oracle     vs FP64 plain oracle
                          (the same cache, read back from the device, looked
                          up by the oracle's restatement of
                          src/cache_performance_renderer.cu)
    delta_db              psnr_cached_fp64_db - psnr_cached_db: what the GPU's
                          arithmetic (fp16 MLP, fp32 marcher and lookups)
                          loses against the FP64 evaluation of the same cached
                          method; <= 0.1 dB is the clause
    cache_vs_plain_db     GPU cached vs GPU plain: the reference's own gate
                          for cached renders (>= 35 dB, src/eval.cu:315-327)

The cache's interpolation error itself (the gap between psnr_plain_db and
psnr_cached_db) belongs to the method, not to the implementation; it is
bounded by the cache-vs-plain gate.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as orc


def pixel_rgb(results: np.ndarray) -> np.ndarray:
    """White-background colour of BaseRayResult rows [..., 4] (rgb, T)."""
    r = np.asarray(results, np.float64)
    return r[..., :3] + r[..., 3:4]


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    return orc.psnr(a, b)


def cached_quality(om: "orc.OracleModel", cam: dict, rows: tuple[int, int], plain_gpu: np.ndarray,
                   cached_gpu: np.ndarray, cache_arrays, cache_cam: dict, threads: int | None = None) -> dict:
    """Quality of one frame over image rows [r0, r1).

    plain_gpu / cached_gpu: full-frame GPU results [H, W, 4];
    cache_arrays: (packed, known, voxels) of the cache the cached frame was
    rendered from (Cache.read()), built at cache_cam."""
    r0, r1 = rows
    W, H = cam["resolution"]
    ref_plain, _, _ = om.render_plain(cam, rows=rows, threads=threads)
    oc = orc.OracleCache(om.cache_dims(W, H), cache_cam)
    oc.load_device_cache(*cache_arrays)
    ref_cached, counts = om.render_cached(cam, oc, rows=rows, threads=threads)
    band = slice(r0, r1)
    p_ref = pixel_rgb(ref_plain[band])
    p_plain = pixel_rgb(plain_gpu[band])
    p_cached = pixel_rgb(cached_gpu[band])
    p_ref_cached = pixel_rgb(ref_cached[band])
    psnr_plain = psnr(p_plain, p_ref)
    psnr_cached = psnr(p_cached, p_ref)
    psnr_cached_fp64 = psnr(p_ref_cached, p_ref)
    hits = int(counts[band][..., 1].sum())
    res = int(counts[band][..., 0].sum())
    return {
        "rows": [int(r0), int(r1)],
        "psnr_plain_db": psnr_plain,
        "psnr_cached_db": psnr_cached,
        "psnr_cached_fp64_db": psnr_cached_fp64,
        "delta_db": psnr_cached_fp64 - psnr_cached,
        "cache_vs_plain_db": psnr(p_cached, p_plain),
        "max_abs_plain": float(np.abs(p_plain - p_ref).max()),
        "max_abs_cached_vs_fp64_cached": float(np.abs(p_cached - p_ref_cached).max()),
        "band_coverage": hits / max(1, hits + res),
    }
