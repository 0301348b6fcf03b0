"""The color head with the positional frequency encoding
(freq_encoding_degree 4: NerfNetwork::init, include/nerf_network.h:103; the
encoding of the network's input position appended after the SH inputs,
:55-81,241-246) against the float64 oracle.

The head reads [latents | SH of the direction | sin, cos(pi 2^k p) per axis,
k < 4] (48 inputs); a view-dependent split head also the SH difference to
the initial direction before them (64 inputs).  A resampled row's position is its contracted sample
point; a cache row's is the contracted point at its network-input midpoint
(src/cache_performance_renderer.cu:284-297).  Bit-exact: sample counts,
classification, brick slots and known ranges.  Within tolerance: pixel
colours (max-abs 2e-3).  The paths not built for these heads (mma.sync,
BF16/FP8, 64- and 256-row tiles, adjoint, autotuner) refuse the model with
FVC_ERR_CONFIG."""
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


def _spec(nlvl: int, head_hidden: int = 2, view_dependent: bool = False):
    spec = fmodel.spec_tiny(seed=41, nlvl=nlvl)
    spec.freq_encoding_degree = 4
    spec.head_hidden_layers = head_hidden
    spec.view_dependent = view_dependent
    spec.name = f"{spec.name}_h{head_hidden}"
    return spec


# the view-dependent case is the reference's custom split head with FREQ_ENC_DEGREE 4
# (src/my_fully_fused_mlp.cu:1358-1421): [latents | SH | SH difference | frequency], 64 inputs
@pytest.fixture(scope="module", params=[(1, 2, False), (3, 2, False), (1, 1, False), (1, 1, True), (3, 2, True)],
                ids=["c1", "c3", "c1_head1", "c1_viewdep_head1", "c3_viewdep"])
def freq_model(request):
    d = fmodel.ensure_model(_spec(*request.param))
    return fvc.load_data(d), orc.OracleModel(d, mimic_fp16=True)


def _rotated(cam0, W, H, deg=1.0):
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(deg)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    return fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)


def test_plain_render(freq_model):
    loader, om = freq_model
    assert om.net.freq_deg == 4 and om.net.head_in == (64 if om.view_dependent else 48)
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
    print(f"\nfrequency-encoded head, plain: max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB, samples {ns.sum()}")
    assert ns.sum() > 0 and err <= COLOR_ATOL
    # the encoding reaches the colour: the same render with the encoding's weights' inputs at zero differs
    no_freq = orc.OracleModel(loader.nerf_network.path, mimic_fp16=True)
    no_freq.net.freq_deg = 0
    ref0, _, _ = no_freq.render_plain(cam)
    assert np.abs(ref0 - ref).max() > 10 * COLOR_ATOL


@pytest.mark.parametrize("fused", [True, False], ids=["march_classifies", "classify_pass"])
def test_cache_build_and_cached_render(freq_model, fused):
    loader, om = freq_model
    if om.view_dependent and not fused:
        pytest.skip("view-dependent models always take the classification pass")
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.set_fused_classify(fused)
    r.setCacheSettings(fvc.default_cache_settings())
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    packed, known, vox = c1.read()
    oc = om.cache_build(cam0)
    np.testing.assert_array_equal(packed.ravel(), oc.packed_index)
    np.testing.assert_array_equal(known.ravel().view(np.uint32), oc.known_ranges.view(np.uint32))
    r.swapCache()
    cam1 = _rotated(cam0, W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    oc.load_device_cache(packed, known, vox)
    ref, counts = om.render_cached(cam1, oc)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    np.testing.assert_array_equal(buf.ray_counts[..., 2][live], counts[..., 2][live])
    err = np.abs(buf.results - ref).max()
    hit = counts[..., 1].sum() / max(1, counts[..., :2].sum())
    p = psnr(buf.results[..., :3] + buf.results[..., 3:], ref[..., :3] + ref[..., 3:])
    print(f"\nfrequency-encoded head, cached: hit {hit:.3f}, max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB")
    assert hit > 0.3 and err <= COLOR_ATOL


def test_basic_cache_renderer(freq_model):
    loader, om = freq_model
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CacheBasicRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings(fvc.DENSITY, fvc.LINEAR))
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    packed, known, vox = c1.read()
    r.swapCache()
    oc = om.cache_build(cam0).render_as_basic(fvc.DENSITY, fvc.LINEAR, 1, 1, 1)
    oc.load_device_cache(packed, known, vox)
    cam1 = _rotated(cam0, W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    ref, counts = om.render_cached(cam1, oc)
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    err = np.abs(buf.results - ref).max()
    print(f"\nfrequency-encoded head, basic cached: max-abs {err:.2e}")
    assert err <= COLOR_ATOL


def test_paths_not_built_refuse_the_model():
    d = fmodel.ensure_model(_spec(1))
    loader = fvc.load_data(d)
    cam = small_camera(1001, 16, 16)
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    for setup, undo in ((lambda: r.set_network_path(False), lambda: r.set_network_path(True)),
                        (lambda: r.set_precision(fvc.PerformanceRenderer.BF16), lambda: r.set_precision(fvc.PerformanceRenderer.FP16)),
                        (lambda: r.set_tiling(64, 0), lambda: r.set_tiling(128, 0)),
                        (lambda: r.set_tiling(256, 0), lambda: r.set_tiling(128, 0))):
        setup()
        with pytest.raises(fvc._lib.FvcError) as e:
            r.render(info, fvc.RenderBuffer((16, 16)))
        assert e.value.code == FVC_ERR_CONFIG and "frequency encoding" in str(e.value)
        undo()
    r.render(info, fvc.RenderBuffer((16, 16)))  # the built path still renders
    with pytest.raises(fvc._lib.FvcError) as e:
        fvc.Gradients(loader.nerf_network)
    assert e.value.code == FVC_ERR_CONFIG
    with pytest.raises(fvc._lib.FvcError) as e:
        r.autotune([info, info])
    assert e.value.code == FVC_ERR_CONFIG
