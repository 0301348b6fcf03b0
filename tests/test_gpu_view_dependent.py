"""The view-dependent split network (NerfNetwork::init_viewdep,
include/nerf_network.h:120-158; loaded when the model has mlp_first_head,
src/loader.cu:251-262) against the oracle.

The latents come from a first head on [density outputs | SH of an initial
direction]. For a plain or resampled sample that direction is the ray's own,
so the head's SH-difference input is zero. The cache build uses its own rays'
directions. A cache sample's initial direction points from the cache camera to
the sample (src/cache_performance_renderer.cu:290-312).
Bit-exact: sample counts, classification, brick slots and known ranges.
Within tolerance: pixel colours (max-abs 2e-3 against the float64 oracle).
The paths not built for these models (mma.sync, BF16/FP8, adjoint, the
autotuner) refuse them with FVC_ERR_CONFIG; batches are checked in
test_gpu_batch.py."""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import psnr, small_camera

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3
FVC_ERR_CONFIG = 2


def _spec(nlvl: int, head_hidden: int = 2, first_latent_is_density: bool = False):
    spec = fmodel.spec_tiny(seed=31, nlvl=nlvl)
    spec.view_dependent = True
    spec.head_hidden_layers = head_hidden
    spec.first_latent_is_density = first_latent_is_density
    spec.name = f"{spec.name}_h{head_hidden}{'_fld' if first_latent_is_density else ''}"
    return spec


@pytest.fixture(scope="module", params=[(1, 2, False), (3, 2, False), (1, 1, False), (1, 2, True)],
                ids=["c1", "c3", "c1_head1", "c1_density_first"])
def vd_model(request):
    d = fmodel.ensure_model(_spec(*request.param))
    return fvc.load_data(d), orc.OracleModel(d, mimic_fp16=True)


def _rotated(cam0, W, H, deg=1.0):
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(deg)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    return fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)


def _check_latents(vox, oc):
    """the voxels' 8 latents (the first head's outputs on the build rays'
    directions) against the oracle's, within fp16 rounding"""
    n = oc.n_bricks_set
    lat = vox[:n, :, 4:8].copy().view(np.float16).astype(np.float32).reshape(n, 512, 8)
    olat = oc.vox_latents[:n * 512 * 8].view(np.float16).astype(np.float32).reshape(n, 512, 8)
    assert n > 0 and np.abs(lat - olat).max() < 2e-3


def test_plain_render(vd_model):
    loader, om = vd_model
    W, H = 48, 40
    cam = small_camera(1001, W, H)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.resizeRenderbuffers((W, H))
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
    ref, ns, nst = om.render_plain(cam)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], ns)
    np.testing.assert_array_equal(buf.ray_counts[..., 3][live], nst[live])
    err = np.abs(buf.results - ref).max()
    p = psnr(buf.results[..., :3] + buf.results[..., 3:], ref[..., :3] + ref[..., 3:])
    print(f"\nview-dependent plain: max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB, samples {ns.sum()}")
    assert ns.sum() > 0 and err <= COLOR_ATOL


def test_cache_build_and_cached_render(vd_model):
    loader, om = vd_model
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings(fvc.DENSITY_INTERMEDIATES if om.net.latent_offset == 0 else fvc.DENSITY))
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    packed, known, vox = c1.read()
    variant = fvc.DENSITY_INTERMEDIATES if om.net.latent_offset == 0 else fvc.DENSITY
    oc = om.cache_build(cam0, variant=variant)
    np.testing.assert_array_equal(packed.ravel(), oc.packed_index)
    np.testing.assert_array_equal(known.ravel().view(np.uint32), oc.known_ranges.view(np.uint32))
    _check_latents(vox, oc)
    r.swapCache()
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
    p = psnr(buf.results[..., :3] + buf.results[..., 3:], ref[..., :3] + ref[..., 3:])
    print(f"\nview-dependent cached: hit {hit:.3f}, max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB")
    assert hit > 0.3 and err <= COLOR_ATOL


def test_paths_not_built_refuse_the_model():
    d = fmodel.ensure_model(_spec(1))
    loader = fvc.load_data(d)
    cam = small_camera(1001, 16, 16)
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.set_network_path(False)
    with pytest.raises(fvc._lib.FvcError) as e:
        r.render(info, fvc.RenderBuffer((16, 16)))
    assert e.value.code == FVC_ERR_CONFIG and "view-dependent" in str(e.value)
    r.set_network_path(True)
    r.set_precision(fvc.PerformanceRenderer.BF16)
    with pytest.raises(fvc._lib.FvcError) as e:
        r.render(info, fvc.RenderBuffer((16, 16)))
    assert e.value.code == FVC_ERR_CONFIG
    r.set_precision(fvc.PerformanceRenderer.FP16)
    r.render(info, fvc.RenderBuffer((16, 16)))  # the built path still renders
    with pytest.raises(fvc._lib.FvcError) as e:
        fvc.Gradients(loader.nerf_network)
    assert e.value.code == FVC_ERR_CONFIG
    with pytest.raises(fvc._lib.FvcError) as e:
        r.autotune([info, info])  # its candidates include the mma.sync path
    assert e.value.code == FVC_ERR_CONFIG


def test_per_ray_fill(vd_model):
    """CacheRenderer::initCache (src/cache_renderer.cu:848-928): the first head
    runs on each row's own ray direction (:899)."""
    loader, om = vd_model
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    variant = fvc.DENSITY_INTERMEDIATES if om.net.latent_offset == 0 else fvc.DENSITY
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings(variant))
    r.initCache(fvc.raymarch_info(cam0, loader.stepsize_info))
    packed, known, vox = c1.read()
    oc = om.cache_build_per_ray(cam0, variant=variant)
    np.testing.assert_array_equal(packed.ravel(), oc.packed_index)
    np.testing.assert_array_equal(known.ravel().view(np.uint32), oc.known_ranges.view(np.uint32))
    _check_latents(vox, oc)
    r.swapCache()
    cam1 = _rotated(cam0, W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    ref, counts = om.render_cached(cam1, oc)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    err = np.abs(buf.results - ref).max()
    hit = counts[..., 1].sum() / max(1, counts[..., :2].sum())
    print(f"\nview-dependent per-ray fill: hit {hit:.3f}, max-abs {err:.2e}")
    assert hit > 0.1 and err <= COLOR_ATOL


def test_basic_cache_renderer(vd_model):
    """CacheBasicRenderer (src/cache_basic_renderer.cu): the cache rows' initial
    direction is taken at the step midpoint (:86-87,198)."""
    loader, om = vd_model
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    variant = fvc.DENSITY_INTERMEDIATES if om.net.latent_offset == 0 else fvc.DENSITY
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CacheBasicRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings(variant, fvc.LINEAR))
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    r.swapCache()
    oc = om.cache_build(cam0, variant=variant).render_as_basic(variant, fvc.LINEAR, 1, 1, 1)
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
    p = psnr(buf.results[..., :3] + buf.results[..., 3:], ref[..., :3] + ref[..., 3:])
    print(f"\nview-dependent basic cached: hit {hit:.3f}, max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB")
    assert hit > 0.3 and err <= COLOR_ATOL
