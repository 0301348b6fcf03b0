"""GPU parity on the benchmark's own scenes, against the float64 oracle.

  - the 256x256 plain workload (one cascade over [-1.5,1.5]^3, 2^16 entries
    per level, cone 0, step 3/1024), full frame;
  - the 1920x1080 cached workload (three cascades over [-6,6]^3 with the
    L-infinity contraction, 2^19 entries per level, cone 1/256, step
    sqrt(3)/1024): a band of rows of the plain frame and of a cached frame
    rendered from a cache built one path step (0.5 degrees + 0.01 units)
    earlier, with the device's cache read back into the oracle;
  - the quality clause of the cached path (dPSNR <= 0.1 dB against the
    float64 oracle, cache vs plain >= 35 dB as src/eval.cu:315-327) on the
    same scene at 480x270, whole frame.

Counts are bit-exact: per-ray samples (and steps on rays that did not
terminate), and the cached render's resample / cache / dropped counts.
Colours: max-abs <= 2e-3 on BaseRayResult (rgb, T).
"""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from oracle import quality as oq

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3      # max-abs on BaseRayResult against the float64 oracle
DELTA_PSNR_DB = 0.1    # quality clause of the cached path
CACHE_VS_PLAIN_DB = 35.0


@pytest.fixture(scope="module")
def config1():
    spec = fmodel.spec_config1()
    d = fmodel.ensure_model(spec)
    return spec, fvc.load_data(d), orc.OracleModel(d)


@pytest.fixture(scope="module")
def config2():
    spec = fmodel.spec_config2()
    d = fmodel.ensure_model(spec)
    return spec, fvc.load_data(d), orc.OracleModel(d)


def _plain(loader, cam):
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.resizeRenderbuffers(cam["resolution"])
    buf = fvc.RenderBuffer(cam["resolution"])
    r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
    return r, buf


def _cached(loader, cam_build, cam_render):
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache(cam_render["resolution"], loader.stepsize_info)
    r.resizeRenderbuffers(cam_render["resolution"])
    r.setCacheSettings(fvc.default_cache_settings())
    r.initCacheBlockwise(fvc.raymarch_info(cam_build, loader.stepsize_info))
    r.swapCache()
    buf = fvc.RenderBuffer(cam_render["resolution"])
    r.render(fvc.raymarch_info(cam_render, loader.stepsize_info), buf)
    return r, buf, c1


def test_config1_full_frame_matches_oracle(config1):
    spec, loader, om = config1
    cam = fcam.seeded_camera(spec.seed, width=256, height=256)
    r, buf = _plain(loader, cam)
    ref, ns, nst = om.render_plain(cam)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], ns)
    np.testing.assert_array_equal(buf.ray_counts[..., 3][live], nst[live])
    err = float(np.abs(buf.results - ref).max())
    p = oq.psnr(oq.pixel_rgb(buf.results), oq.pixel_rgb(ref))
    # 8-bit image: a colour within rounding of a quantisation boundary may land one step away
    img = orc.composite_image(ref)
    diff = np.abs(buf.image.astype(np.int32) - img.astype(np.int32))
    print(f"\nconfig 1 256x256: samples {int(ns.sum())}, max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB, "
          f"8-bit pixels off by one {int((diff > 0).sum())}")
    assert err <= COLOR_ATOL
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-2
    assert r._render_stats.guard_flags == 0


def test_config2_row_band_plain_and_cached_match_oracle(config2):
    spec, loader, om = config2
    cams = fcam.rotation_path(spec.seed, n_frames=2, width=1920, height=1080)
    rows = (536, 544)
    band = slice(*rows)
    _, plain = _plain(loader, cams[1])
    ref, ns, nst = om.render_plain(cams[1], rows=rows)
    live = ref[band][..., 3] >= 1e-4
    np.testing.assert_array_equal(plain.ray_counts[band][..., 0], ns[band])
    np.testing.assert_array_equal(plain.ray_counts[band][..., 3][live], nst[band][live])
    err = float(np.abs(plain.results[band] - ref[band]).max())
    assert err <= COLOR_ATOL, err

    r, cached, c1 = _cached(loader, cams[0], cams[1])
    arrays = c1.read()
    oc = orc.OracleCache(om.cache_dims(1920, 1080), cams[0])
    oc.load_device_cache(*arrays)
    cref, counts = om.render_cached(cams[1], oc, rows=rows)
    clive = cref[band][..., 3] >= 1e-4
    np.testing.assert_array_equal(cached.ray_counts[band][..., 0], counts[band][..., 0])  # resample
    np.testing.assert_array_equal(cached.ray_counts[band][..., 1], counts[band][..., 1])  # cache
    np.testing.assert_array_equal(cached.ray_counts[band][..., 2][clive], counts[band][..., 2][clive])  # dropped
    cerr = float(np.abs(cached.results[band] - cref[band]).max())
    hits = counts[band][..., 1].sum() / max(1, counts[band][..., :2].sum())
    print(f"\nconfig 2 rows {rows}: plain max-abs {err:.2e}, cached max-abs {cerr:.2e}, band coverage {hits:.3f}")
    assert cerr <= COLOR_ATOL, cerr


def test_config2_quality_clause(config2):
    """dPSNR <= 0.1 dB against the float64 oracle and cache vs plain >= 35 dB
    on the cached workload's scene at 480x270, frame 1 of the camera path
    rendered from the cache built at frame 0."""
    spec, loader, om = config2
    W, H = 480, 270
    cams = fcam.rotation_path(spec.seed, n_frames=2, width=W, height=H)
    _, plain = _plain(loader, cams[1])
    _, cached, c1 = _cached(loader, cams[0], cams[1])
    q = oq.cached_quality(om, cams[1], (0, H), plain.results, cached.results, c1.read(), cams[0])
    print("\nquality " + ", ".join(f"{k} {v:.4g}" if isinstance(v, float) else f"{k} {v}" for k, v in q.items()))
    assert q["delta_db"] <= DELTA_PSNR_DB, q
    assert q["cache_vs_plain_db"] >= CACHE_VS_PLAIN_DB, q
    assert q["max_abs_plain"] <= COLOR_ATOL and q["max_abs_cached_vs_fp64_cached"] <= COLOR_ATOL, q
