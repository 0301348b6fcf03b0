"""The 8-level x 4-feature hash grid (instant-ngp's NeRF default; the
reference loads any tiny-cuda-nn grid, src/loader.cu:146-230) against the
float64 oracle: network outputs, plain renders on every network path and tile
height, a cached render; an instant-ngp snapshot with that grid exports and
renders; the adjoint refuses it (built for 16 levels of 2 features)."""
import dataclasses

import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import small_camera

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3


def _spec(nlvl):
    s = fmodel.spec_tiny(seed=41, nlvl=nlvl)
    return dataclasses.replace(s, name=f"{s.name}_f4", n_levels=8, F=4, per_level_scale=2.0)


@pytest.fixture(scope="module", params=[1, 3], ids=["c1", "c3"])
def model(request):
    d = fmodel.ensure_model(_spec(request.param))
    return fvc.load_data(d), orc.OracleModel(d), d


def test_network_outputs_match_oracle(model):
    loader, om, _ = model
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 1, (4000, 3)).astype(np.float32)
    dirs = rng.uniform(0, 1, (4000, 3)).astype(np.float32)
    got = loader.nerf_network.inference(pos, dirs)
    ref = om.inference(pos, dirs)
    assert np.abs(got - ref).max() <= 2e-3


@pytest.mark.parametrize("path", ["tc128", "tc64", "tc256", "mma"])
def test_plain_render_matches_oracle(model, path):
    loader, om, _ = model
    cam = small_camera(1001, 48, 40)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    if path == "mma":
        r.set_network_path(False)
    else:
        r.set_tiling(int(path[2:]), 0)
    buf = fvc.RenderBuffer((48, 40))
    r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
    ref, ns, nst = om.render_plain(cam)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], ns)
    np.testing.assert_array_equal(buf.ray_counts[..., 3][live], nst[live])
    assert float(np.abs(buf.results - ref).max()) <= COLOR_ATOL
    assert ns.sum() > 1000


def test_cached_render_matches_oracle(model):
    loader, om, _ = model
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings())
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    r.swapCache()
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(1.0)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    cam1 = fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    oc = orc.OracleCache(om.cache_dims(W, H), cam0)
    oc.load_device_cache(*c1.read())
    ref, counts = om.render_cached(cam1, oc)
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    assert counts[..., 1].sum() > 0
    assert float(np.abs(buf.results - ref).max()) <= COLOR_ATOL


def test_adjoint_refuses_the_four_feature_grid(model):
    loader, _, _ = model
    with pytest.raises(fvc._lib.FvcError):
        fvc.Gradients(loader.nerf_network)
