"""Failure paths, made to happen on the host or by a wait that nothing ends
(never by faulting the GPU): the kernels' bounded device wait gives up and
reports it; an allocation that fails returns FVC_ERR_OOM and leaves the
renderer usable; a frame in which no ray hits the scene; a blockwise cache
build that demands more bricks than the reference sizing reserves."""
import ctypes as C

import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import _lib as L
from frustumvolumecaching_gb300 import camera as fcam
from oracle import oracle as orc
from tests.helpers import small_camera, tiny_model

pytestmark = pytest.mark.gpu

FVC_ERR_OOM, FVC_ERR_TIMEOUT = 3, 5


@pytest.fixture(scope="module")
def loader():
    return fvc.load_data(tiny_model(7, 1))


def _plain(loader, cam):
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    buf = fvc.RenderBuffer(cam["resolution"])
    r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
    return r, buf


def test_bounded_wait_gives_up_and_the_context_stays_usable(loader):
    waited = C.c_double()
    rc = L.load().fvc_selftest_wait_timeout(5.0, C.byref(waited))
    assert rc == FVC_ERR_TIMEOUT, L.load().fvc_last_error()
    assert b"gave up" in L.load().fvc_last_error()
    assert 4.0 <= waited.value < 500.0
    cam = small_camera(1001, 32, 24)
    _, buf = _plain(loader, cam)
    assert buf.ray_counts[..., 0].sum() > 0 and np.isfinite(buf.results).all()


def test_injected_allocation_failure_leaves_the_renderer_usable(loader):
    lib = L.load()
    cam_a, cam_b = small_camera(1001, 32, 24), small_camera(1001, 48, 40)
    r, _ = _plain(loader, cam_a)
    buf = fvc.RenderBuffer((48, 40))
    try:
        assert lib.fvc_debug_fail_allocation(2) == 0  # the 3rd allocation of the resize fails
        with pytest.raises(L.FvcError) as e:
            r.render(fvc.raymarch_info(cam_b, loader.stepsize_info), buf)
        assert e.value.code == FVC_ERR_OOM and "injected" in str(e.value)
    finally:
        lib.fvc_debug_fail_allocation(-1)
    r.render(fvc.raymarch_info(cam_b, loader.stepsize_info), buf)
    _, ref = _plain(loader, cam_b)
    np.testing.assert_array_equal(buf.results, ref.results)
    np.testing.assert_array_equal(buf.ray_counts, ref.ray_counts)


def test_frame_in_which_no_ray_hits_the_scene(loader):
    cam = small_camera(1001, 32, 24)
    c2w = np.asarray(cam["cam2world"], np.float64).copy()
    c2w[:, :3] = -c2w[:, :3]  # look away from the scene box
    c2w[:, 0] = -c2w[:, 0]    # keep a right-handed frame
    away = fcam.camera_dict(c2w, 32, 24)
    r, buf = _plain(loader, away)
    assert (buf.ray_counts[..., :3] == 0).all()  # no sample (a box behind the camera still clips to an empty range)
    np.testing.assert_array_equal(buf.results[..., 3], 1.0)
    assert (buf.image[..., :3] == 255).all()
    assert r._render_stats.n_samples == 0 and r._render_stats.guard_flags == 0
    # a cache built from that view holds no brick and renders the same frame
    c0, c1 = fvc.Cache(), fvc.Cache()
    rc = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    rc.resizeCache((32, 24), loader.stepsize_info)
    rc.resizeRenderbuffers((32, 24))
    rc.setCacheSettings(fvc.default_cache_settings())
    rc.initCacheBlockwise(fvc.raymarch_info(away, loader.stepsize_info))
    assert rc._init_stats.n_bricks_set == 0
    rc.swapCache()
    b2 = fvc.RenderBuffer((32, 24))
    rc.render(fvc.raymarch_info(away, loader.stepsize_info), b2)
    np.testing.assert_array_equal(b2.results, buf.results)


def test_blockwise_build_overflow_matches_the_oracle(loader):
    """320x240 demands more bricks than the 16,384 slots the reference sizing
    reserves: tiles stop where their brick finds no slot, as in
    accumulateNew_cache_init_second_kernel (src/cache_renderer.cu:419-426,
    518-527)."""
    om = orc.OracleModel(tiny_model(7, 1))
    cam = small_camera(1001, 320, 240)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((320, 240), loader.stepsize_info)
    r.resizeRenderbuffers((320, 240))
    r.setCacheSettings(fvc.default_cache_settings())
    r.initCacheBlockwise(fvc.raymarch_info(cam, loader.stepsize_info))
    packed, known, _ = c1.read()
    oc = om.cache_build(cam)
    st = r._init_stats
    assert oc.n_demanded > oc.n_bricks_set == 16384
    assert st.n_bricks_demanded == oc.n_demanded and st.n_bricks_set == oc.n_bricks_set
    np.testing.assert_array_equal(packed.ravel(), oc.packed_index)
    np.testing.assert_array_equal(known.ravel().view(np.uint32), oc.known_ranges.view(np.uint32))
