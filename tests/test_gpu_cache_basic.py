"""GPU parity of the basic cache renderer (CacheBasicRenderer,
src/cache_basic_renderer.cu) against the oracle: the cache decides by the
voxel's isset flag, every CacheSettings field applies (interpolation
function, density variant, reweighting of the intermediates, inter-brick
interpolation), and cache samples composite with their looked-up density.
Bit-exact: per-ray resample / cache / dropped counts.  Within tolerance:
pixel colours (max-abs 2e-3 against the float64 oracle)."""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import psnr, small_camera, tiny_model

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3


def _fld_model(seed: int, nlvl: int) -> str:
    spec = fmodel.spec_tiny(seed=seed, nlvl=nlvl)
    spec.name = f"{spec.name}_fld"
    spec.first_latent_is_density = True
    return fmodel.ensure_model(spec)


@pytest.fixture(scope="module")
def models():
    return {k: (fvc.load_data(d), orc.OracleModel(d))
            for k, d in (("lo1", tiny_model(7, 1)), ("lo1_c3", tiny_model(9, 3)), ("lo0", _fld_model(7, 1)))}


def _rotated(cam0, W, H, deg=1.0):
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(deg)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    return fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)


CASES = [  # model, variant, interpolation, reweight, keep first, inter-brick
    ("lo1", fvc.DENSITY, fvc.LINEAR, 1, 1, 1),
    ("lo1", fvc.DENSITY, fvc.LINEAR, 1, 1, 0),
    ("lo1", fvc.DENSITY, fvc.LINEAR, 0, 0, 1),
    ("lo1", fvc.DENSITY, fvc.SMOOTHSTEP, 1, 0, 1),
    ("lo1", fvc.DENSITY, fvc.NEAREST, 1, 1, 1),
    ("lo1", fvc.ALPHA, fvc.LINEAR, 1, 1, 1),
    ("lo1", fvc.ALPHA_INTERMEDIATES, fvc.SMOOTHERSTEP, 1, 1, 1),
    ("lo1_c3", fvc.DENSITY, fvc.LINEAR, 1, 1, 1),
    ("lo0", fvc.DENSITY_INTERMEDIATES, fvc.LINEAR, 1, 1, 1),
    ("lo0", fvc.INTERMEDIATES, fvc.LINEAR, 1, 0, 1),
]


@pytest.mark.parametrize("tcgen05", [False, True], ids=["mma_sync", "tcgen05"])
@pytest.mark.parametrize("key,variant,interp,reweight,keep_first,inter_brick", CASES)
def test_basic_cache_renderer_parity(models, key, variant, interp, reweight, keep_first, inter_brick, tcgen05):
    loader, om = models[key]
    W, H = (48, 40) if key.endswith("c3") else (64, 48)
    cam0 = small_camera(1001, W, H)
    settings = fvc.default_cache_settings(variant, interp)
    settings.reweight_intermediates, settings.disable_reweighting_first_intermediate = reweight, keep_first
    settings.use_inter_brick_interpolation = inter_brick
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CacheBasicRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(settings)
    r.set_network_path(tcgen05)
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    r.swapCache()
    oc = om.cache_build(cam0, variant=variant).render_as_basic(variant, interp, reweight, keep_first, inter_brick)
    cam1 = _rotated(cam0, W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    ref, counts = om.render_cached(cam1, oc)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    np.testing.assert_array_equal(buf.ray_counts[..., 2][live], counts[..., 2][live])
    assert np.isfinite(buf.results).all()
    err = np.abs(buf.results - ref).max()
    hit = counts[..., 1].sum() / max(1, counts[..., :2].sum())
    p = psnr(buf.results[..., :3] + buf.results[..., 3:], ref[..., :3] + ref[..., 3:])
    print(f"\nbasic {key} variant {variant} interp {interp} reweight {reweight}/{keep_first} inter-brick {inter_brick} "
          f"{'tcgen05' if tcgen05 else 'mma.sync'}: hit {hit:.3f}, max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB")
    assert hit > 0.3
    assert err <= COLOR_ATOL


def test_basic_renderer_takes_every_variant_and_refuses_the_adjoint(models):
    loader, _ = models["lo1"]
    cam = small_camera(1001, 16, 16)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CacheBasicRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((16, 16), loader.stepsize_info)
    r.resizeRenderbuffers((16, 16))
    for v in (fvc.DENSITY, fvc.ALPHA, fvc.INTERMEDIATES, fvc.DENSITY_INTERMEDIATES, fvc.ALPHA_INTERMEDIATES):
        r.setCacheSettings(fvc.default_cache_settings(v, fvc.LINEAR))
    r.initCacheBlockwise(fvc.raymarch_info(cam, loader.stepsize_info))
    r.swapCache()
    import torch
    g = fvc.Gradients(loader.nerf_network)
    px = torch.arange(16, dtype=torch.int32, device="cuda")
    tg = torch.zeros((16, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(fvc._lib.FvcError) as e:
        r.render_backward(fvc.raymarch_info(cam, loader.stepsize_info), px, tg, g)
    assert e.value.code == 2
