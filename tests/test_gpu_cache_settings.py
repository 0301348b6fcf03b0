"""GPU parity of the cache settings the cached performance renderer reads
(CacheSettings, include/cache_renderer.h:24-32): the interpolation function
of the trilinear lookup (Linear, Smoothstep, Smootherstep, Nearest;
applyInterpolationFunction, include/raymarch_common.h:393-402) and the
density variants (what a build stores in the voxels' density slot and latent
0, accumulateNew_cache_init_second_kernel, src/cache_renderer.cu:459-507; how
a lookup forms the head input, src/cache_performance_renderer.cu:740-787).

DensityIntermediates is the variant eval picks for a model whose first
latent is the density (src/eval.cu:215-222), e.g. every instant-ngp snapshot.

Bit-exact: slot assignment, isset, per-ray resample / cache counts.  Within
tolerance: voxel densities and latents, pixel colours (max-abs 2e-3 against
the float64 oracle).
"""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import psnr, small_camera, tiny_model

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3  # max-abs pixel tolerance against the float64 oracle


def _fld_model(seed: int, nlvl: int) -> str:
    """A tiny model whose first latent is the density (latent_offset 0)."""
    spec = fmodel.spec_tiny(seed=seed, nlvl=nlvl)
    spec.name = f"{spec.name}_fld"
    spec.first_latent_is_density = True
    return fmodel.ensure_model(spec)


@pytest.fixture(scope="module")
def models():
    out = {}
    for key, d in (("lo1", tiny_model(7, 1)), ("lo1_c3", tiny_model(9, 3)), ("lo0", _fld_model(7, 1)),
                   ("lo0_c3", _fld_model(9, 3))):
        out[key] = (fvc.load_data(d), orc.OracleModel(d))
    return out


def _rotated(cam0, W, H, deg=1.0):
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(deg)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    return fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)


def _setup(loader, cam, settings):
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache(cam["resolution"], loader.stepsize_info)
    r.resizeRenderbuffers(cam["resolution"])
    r.setCacheSettings(settings)
    return r, c0, c1


CASES = [
    ("lo1", fvc.DENSITY, fvc.SMOOTHSTEP),
    ("lo1", fvc.DENSITY, fvc.SMOOTHERSTEP),
    ("lo1", fvc.DENSITY, fvc.NEAREST),
    ("lo1", fvc.ALPHA, fvc.LINEAR),
    ("lo1", fvc.ALPHA_INTERMEDIATES, fvc.LINEAR),
    ("lo1_c3", fvc.DENSITY, fvc.SMOOTHSTEP),
    ("lo0", fvc.DENSITY_INTERMEDIATES, fvc.LINEAR),
    ("lo0", fvc.DENSITY_INTERMEDIATES, fvc.SMOOTHERSTEP),
    ("lo0_c3", fvc.DENSITY_INTERMEDIATES, fvc.LINEAR),
]


@pytest.mark.parametrize("tcgen05", [False, True], ids=["mma_sync", "tcgen05"])
@pytest.mark.parametrize("key,variant,interp", CASES)
def test_cache_settings_parity(models, key, variant, interp, tcgen05):
    loader, om = models[key]
    W, H = (48, 40) if key.endswith("c3") else (64, 48)
    cam0 = small_camera(1001, W, H)
    r, c0, c1 = _setup(loader, cam0, fvc.default_cache_settings(variant, interp))
    r.set_network_path(tcgen05)
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    oc = om.cache_build(cam0, variant=variant, interp=interp)
    # the build: slots and isset bit-exact, the density slot and latents per variant within tolerance
    packed, known, vox = c1.read()
    np.testing.assert_array_equal(packed.ravel(), oc.packed_index)
    n = oc.n_bricks_set
    v = vox[:n].view(np.float32)
    np.testing.assert_array_equal(v[..., 1].ravel(), oc.vox_isset[:n * 512])
    odens = oc.vox_density[:n * 512].reshape(n, 512)
    assert np.abs(v[..., 0] - odens).max() <= 2e-3 * max(1.0, odens.max())
    lat = vox[:n, :, 4:8].copy().view(np.float16).astype(np.float32).reshape(n, 512, 8)
    olat = oc.vox_latents[:n * 512 * 8].view(np.float16).astype(np.float32).reshape(n, 512, 8)
    assert np.abs(lat - olat).max() < 2e-3
    # the render at a view 1 degree away
    r.swapCache()
    cam1 = _rotated(cam0, W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    ref, counts = om.render_cached(cam1, oc)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    np.testing.assert_array_equal(buf.ray_counts[..., 2][live], counts[..., 2][live])
    assert not np.isnan(buf.results).any()
    err = np.abs(buf.results - ref).max()
    p = psnr(buf.results[..., :3] + buf.results[..., 3:], ref[..., :3] + ref[..., 3:])
    hit = counts[..., 1].sum() / max(1, counts[..., :2].sum())
    print(f"\n{key} variant {variant} interp {interp} {'tcgen05' if tcgen05 else 'mma.sync'}: hit {hit:.3f}, "
          f"max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB")
    assert hit > 0.3
    assert err <= COLOR_ATOL


def test_eval_settings_follow_the_model(models):
    """eval's choice (src/eval.cu:215-222) and the combinations refused."""
    lo1, _ = models["lo1"]
    lo0, _ = models["lo0"]
    assert fvc.eval_cache_settings(lo1).interpol_variant == fvc.DENSITY
    assert fvc.eval_cache_settings(lo0).interpol_variant == fvc.DENSITY_INTERMEDIATES
    cam = small_camera(1001, 16, 16)
    for loader, variant in ((lo1, fvc.DENSITY_INTERMEDIATES), (lo0, fvc.DENSITY), (lo0, fvc.ALPHA)):
        r, _, _ = _setup(loader, cam, fvc.default_cache_settings(variant, fvc.LINEAR))
        with pytest.raises(fvc._lib.FvcError) as e:
            r.initCacheBlockwise(fvc.raymarch_info(cam, loader.stepsize_info))
        assert e.value.code == 2  # FVC_ERR_CONFIG
    r, _, _ = _setup(lo1, cam, fvc.default_cache_settings())
    with pytest.raises(fvc._lib.FvcError) as e:
        r.setCacheSettings(fvc.default_cache_settings(fvc.INTERMEDIATES, fvc.LINEAR))
    assert e.value.code == 2
    with pytest.raises(fvc._lib.FvcError) as e:
        r.setCacheSettings(fvc.default_cache_settings(fvc.DENSITY, 7))
    assert e.value.code != 0


@pytest.mark.parametrize("key", ["lo1", "lo1_c3"])
def test_cache_built_at_double_sampling_rate(models, key):
    """The viewer's m_cache_double_sampling_rate (realtime_viewer/src/
    application.cu:73-74): the cache is sized and built with
    StepsizeInfo::changeSamplingRate(2) and the frame renders at the model's
    rate; reprojection and classification use the cache's own step grid."""
    loader, om = models[key]
    W, H = (48, 40) if key.endswith("c3") else (64, 48)
    cam0 = small_camera(1001, W, H)
    cst = fvc.change_sampling_rate(loader.stepsize_info, 2.0, loader.scene_info)
    assert cst.stepsize == np.float32(loader.stepsize_info.stepsize) / np.float32(2)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), cst)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings())
    r.initCacheBlockwise(fvc.raymarch_info(cam0, cst))
    r.swapCache()
    ost = orc.make_steps(om.scene, cst.cone_angle, cst.stepsize, cst.near, cst.far)
    oc = om.cache_build(cam0, steps=ost)
    cam1 = _rotated(cam0, W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    ref, counts = om.render_cached(cam1, oc)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    np.testing.assert_array_equal(buf.ray_counts[..., 2][live], counts[..., 2][live])
    err = np.abs(buf.results - ref).max()
    hit = counts[..., 1].sum() / max(1, counts[..., :2].sum())
    print(f"\n{key} cache at 2x sampling rate: hit {hit:.3f}, max-abs {err:.2e}")
    assert hit > 0.2
    assert err <= COLOR_ATOL
