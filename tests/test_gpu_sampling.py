"""Non-deterministic ray generation on the GPU (RaymarchInfo::deterministic =
false): pixel and start-t jitter over sample_index, depth of field and motion
blur, against the float64 oracle, which shares the sampling arithmetic
(fvc_sampling.h) and is pinned to the reference's code by
test_golden_sampling.py.  Counts bit-exact, colours within 2e-3; the cache
build refuses a non-deterministic RaymarchInfo; progressive accumulation
averages the jittered frames."""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from oracle import oracle as orc
from tests.helpers import small_camera, tiny_model

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3


@pytest.fixture(scope="module")
def model():
    d = tiny_model(7, 1)
    return fvc.load_data(d), orc.OracleModel(d)


def _nd_cam(seed, W, H, spp, **kw):
    cam = dict(small_camera(seed, W, H), deterministic=False, sample_index=spp)
    cam.update(kw)
    return cam


def _render(loader, cam, kind=fvc.PerformanceRenderer):
    r = kind(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    buf = fvc.RenderBuffer(cam["resolution"])
    r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
    return r, buf


CASES = {
    "jitter": {},
    "depth_of_field": {"aperature": 0.04, "focus_z": 3.8},
    "motion_blur": {"motion_blur": True},
    "both": {"aperature": 0.04, "focus_z": 3.8, "motion_blur": True},
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("spp", [0, 7])
def test_nondeterministic_plain_render_matches_oracle(model, case, spp):
    loader, om = model
    W, H = 48, 40
    kw = dict(CASES[case])
    if kw.get("motion_blur"):
        kw["next_cam2world"] = small_camera(1002, W, H)["cam2world"]
    cam = _nd_cam(1001, W, H, spp, **kw)
    r, buf = _render(loader, cam)
    ref, ns, nst = om.render_plain(cam)
    live = ref[..., 3] >= 1e-4
    np.testing.assert_array_equal(buf.ray_counts[..., 0], ns)
    np.testing.assert_array_equal(buf.ray_counts[..., 3][live], nst[live])
    err = float(np.abs(buf.results - ref).max())
    print(f"\n{case} spp {spp}: samples {int(ns.sum())}, max-abs {err:.2e}")
    assert err <= COLOR_ATOL
    # the jitter changes the image against the deterministic render
    det = _render(loader, small_camera(1001, W, H))[1]
    assert not np.array_equal(det.ray_counts, buf.ray_counts)


def test_progressive_average_of_jittered_frames(model):
    loader, _ = model
    W, H = 32, 32
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    buf = fvc.RenderBuffer((W, H))
    prev = None
    for spp in range(4):
        cam = _nd_cam(1001, W, H, spp)
        r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
        expect = orc.composite_image(buf.results, spp, prev)
        np.testing.assert_array_equal(buf.image, expect)
        prev = buf.image.copy()


def test_nondeterministic_cached_render_matches_oracle(model):
    loader, om = model
    W, H = 48, 40
    cam0 = small_camera(1001, W, H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings())
    with pytest.raises(fvc._lib.FvcError):
        r.initCacheBlockwise(fvc.raymarch_info(_nd_cam(1001, W, H, 3), loader.stepsize_info))
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    r.swapCache()
    cam1 = _nd_cam(1001, W, H, 5, aperature=0.03, focus_z=3.8)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam1, loader.stepsize_info), buf)
    oc = orc.OracleCache(om.cache_dims(W, H), cam0)
    oc.load_device_cache(*c1.read())
    ref, counts = om.render_cached(cam1, oc)
    np.testing.assert_array_equal(buf.ray_counts[..., 0], counts[..., 0])
    np.testing.assert_array_equal(buf.ray_counts[..., 1], counts[..., 1])
    assert counts[..., 1].sum() > 0
    assert float(np.abs(buf.results - ref).max()) <= COLOR_ATOL


def test_nondeterministic_batch_matches_single_views(model):
    torch = pytest.importorskip("torch")
    loader, _ = model
    sizes = [(40, 30), (32, 32)]
    cams = [_nd_cam(1300 + i, W, H, 2 + i, aperature=0.02 * i, focus_z=3.9) for i, (W, H) in enumerate(sizes)]
    n = sum(W * H for W, H in sizes)
    res = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    cnt = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.render_batch([fvc.raymarch_info(c, loader.stepsize_info) for c in cams], results=res, ray_counts=cnt)
    r.synchronize()
    res, cnt = res.cpu().numpy(), cnt.cpu().numpy()
    off = 0
    for cam, (W, H) in zip(cams, sizes):
        _, buf = _render(loader, cam)
        np.testing.assert_array_equal(res[off:off + W * H], buf.results.reshape(-1, 4))
        np.testing.assert_array_equal(cnt[off:off + W * H], buf.ray_counts.reshape(-1, 4))
        off += W * H


def test_depth_of_field_without_focus_is_refused(model):
    loader, _ = model
    cam = _nd_cam(1001, 16, 16, 1, aperature=0.1, focus_z=0.0)
    with pytest.raises(fvc._lib.FvcError):
        _render(loader, cam)
