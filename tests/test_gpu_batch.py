"""Batched views in one CUDA-graph launch (fvc_render_batch).

The device-side loop renders each ray exactly as the per-view render does,
so a batch of views of different resolutions must reproduce the single-view
renders on the same network path bit for bit (results, ray counts, image),
whatever the marching batch.  Also checked: a second
batch with new cameras reuses the graph and is still exact, the autotuner
returns a valid configuration, and the statistics report the device loop.
"""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import model as fmodel
from tests.helpers import small_camera, tiny_model

pytestmark = pytest.mark.gpu

SIZES = [(40, 30), (64, 48), (32, 32)]


def _views(seed0):
    return [small_camera(seed0 + i, W, H) for i, (W, H) in enumerate(SIZES)]


def _single(loader, cams, tcgen05=True):
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.set_network_path(tcgen05)
    out = []
    for c in cams:
        buf = fvc.RenderBuffer(c["resolution"])
        r.render(fvc.raymarch_info(c, loader.stepsize_info), buf)
        out.append(buf)
    return out


def _batch(torch, r, loader, cams, tune=False):
    n = sum(W * H for W, H in (c["resolution"] for c in cams))
    res = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    cnt = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    img = torch.zeros((n, 4), dtype=torch.uint8, device="cuda")
    infos = [fvc.raymarch_info(c, loader.stepsize_info) for c in cams]
    tuned = r.autotune(infos, image=img, results=res, ray_counts=cnt) if tune else None
    r.render_batch(infos, image=img, results=res, ray_counts=cnt)
    r.synchronize()
    return res.cpu().numpy(), cnt.cpu().numpy(), img.cpu().numpy(), tuned


def _check(single, res, cnt, img):
    off = 0
    for buf in single:
        H, W = buf.results.shape[:2]
        n = W * H
        np.testing.assert_array_equal(res[off:off + n], buf.results.reshape(-1, 4))
        np.testing.assert_array_equal(cnt[off:off + n], buf.ray_counts.reshape(-1, 4))
        np.testing.assert_array_equal(img[off:off + n], buf.image.reshape(-1, 4))
        off += n


def _model(kind):
    if kind == "view_dependent":  # the split head (mlp_first_head)
        spec = fmodel.spec_tiny(seed=31)
        spec.view_dependent, spec.name = True, f"{spec.name}_h2"
        return fvc.load_data(fmodel.ensure_model(spec))
    return fvc.load_data(tiny_model(7, 1))


@pytest.mark.parametrize("kind", ["density_head", "view_dependent"])
def test_batch_matches_single_views_and_reuses_graph(kind):
    torch = pytest.importorskip("torch")
    loader = _model(kind)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    for seed0 in (1200, 1300):  # the second batch changes only the cameras: same graph
        cams = _views(seed0)
        res, cnt, img, _ = _batch(torch, r, loader, cams)
        _check(_single(loader, cams), res, cnt, img)
    st = r._render_stats
    assert st.n_rounds >= 2 and st.n_launches >= 1 + 9 * (st.n_rounds // 2)
    assert st.guard_flags == 0


def test_autotune_picks_a_valid_configuration():
    torch = pytest.importorskip("torch")
    loader = fvc.load_data(tiny_model(7, 1))
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    cams = _views(1400)
    res, cnt, img, tuned = _batch(torch, r, loader, cams, tune=True)
    # the default space is the batched workload's: tcgen05 tiles {64, 128, 256} x batches 2^16..2^20 x steps {16, 64}
    assert tuned.n_candidates == 30
    assert tuned.steps_per_iter in (16, 64)
    assert tuned.m_tile in (64, 128, 256) and tuned.batch_rows in [1 << k for k in (16, 17, 18, 19, 20)]
    assert tuned.ms > 0 and tuned.rows_per_iteration > 0
    _check(_single(loader, cams), res, cnt, img)
    # a space of the caller's: the mma.sync tile and a batch beyond 2^20 are candidates too
    r.set_autotune_space([32, 128], [1 << 22], [16])
    res, cnt, img, tuned = _batch(torch, r, loader, cams, tune=True)
    assert tuned.n_candidates == 2 and tuned.m_tile in (32, 128) and tuned.batch_rows == 1 << 22 and tuned.steps_per_iter == 16
    # the batch ran with the winner's network path: compare with single views on the same path
    _check(_single(loader, cams, tcgen05=tuned.m_tile != 32), res, cnt, img)
    for bad in (([96], [1 << 16], [16]), ([128], [100], [16]), ([128], [1 << 16], [6]), ([], [1 << 16], [16])):
        with pytest.raises(RuntimeError):
            r.set_autotune_space(*bad)


TILINGS = [(64, 0), (256, 0), (128, 1 << 16), (64, 1 << 17), (256, 1 << 20), (128, 1024)]


@pytest.mark.parametrize("spec_name", ["tiny", "config1"])
def test_tile_heights_and_compaction_batches_are_exact(spec_name):
    """The tcgen05 network on 64- and 256-row tiles and any compaction batch
    give the default render (128-row tiles, batch = row capacity) bit for bit:
    a row's arithmetic does not depend on its tile or sub-iteration."""
    if spec_name == "tiny":
        loader = fvc.load_data(tiny_model(7, 1))
    else:
        loader = fvc.load_data(fmodel.ensure_model(fmodel.spec_config1()))
    cam = small_camera(1601, 96, 80)
    ref = _single(loader, [cam])[0]
    assert ref.ray_counts[..., 0].sum() > 1000
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    for m, b in TILINGS:
        r.set_tiling(m, b)
        buf = fvc.RenderBuffer(cam["resolution"])
        r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
        np.testing.assert_array_equal(buf.results, ref.results, err_msg=f"tile {m} batch {b}")
        np.testing.assert_array_equal(buf.ray_counts, ref.ray_counts, err_msg=f"tile {m} batch {b}")
        assert r._render_stats.guard_flags == 0
    with pytest.raises(fvc._lib.FvcError):
        r.set_tiling(32, 0)
    with pytest.raises(fvc._lib.FvcError):
        r.set_tiling(128, 100)


@pytest.mark.parametrize("m_tile", [64, 128, 256])
def test_batch_of_mixed_resolutions_matches_oracle(m_tile):
    """A batch of views of different resolutions over the 256x256 workload's
    scene (2^16 entries per level) against the float64 oracle, view by view:
    per-ray sample counts exact, steps exact on rays that did not terminate,
    colours within 2e-3."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as orc

    spec = fmodel.spec_config1()
    d = fmodel.ensure_model(spec)
    loader = fvc.load_data(d)
    om = orc.OracleModel(d)
    sizes = [(160, 120), (72, 40), (128, 128), (96, 54)]
    cams = [small_camera(1700 + i, W, H) for i, (W, H) in enumerate(sizes)]
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.set_tiling(m_tile, 1 << 16)
    res, cnt, _, _ = _batch(torch, r, loader, cams)
    off = 0
    for cam, (W, H) in zip(cams, sizes):
        n = W * H
        ref, ns, nst = om.render_plain(cam)
        got_r = res[off:off + n].reshape(H, W, 4)
        got_c = cnt[off:off + n].reshape(H, W, 4)
        live = ref[..., 3] >= 1e-4
        np.testing.assert_array_equal(got_c[..., 0], ns)
        np.testing.assert_array_equal(got_c[..., 3][live], nst[live])
        assert float(np.abs(got_r - ref).max()) <= 2e-3
        off += n
    assert r._render_stats.guard_flags == 0


@pytest.mark.parametrize("kind", ["density_head", "view_dependent"])
def test_batch_with_per_view_caches_matches_single_cached_renders(kind):
    """Each view of a batch renders against its own frustum cache (built at
    the view's pose; rendered from a pose rotated by 1 degree): the batch must
    reproduce the per-view cached renders bit for bit."""
    torch = pytest.importorskip("torch")
    from frustumvolumecaching_gb300 import camera as fcam

    loader = _model(kind)
    cams0 = _views(1500)
    a = np.radians(1.0)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    cams1 = []
    for c in cams0:
        m = np.asarray(c["cam2world"], np.float64)
        W, H = c["resolution"]
        cams1.append(fcam.camera_dict(np.concatenate([R @ m[:, :3], (R @ m[:, 3])[:, None]], axis=1), W, H))
    caches = [fvc.Cache() for _ in cams0]
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network,
                                     caches[0], caches[0])
    r.setCacheSettings(fvc.default_cache_settings())
    for c, cam in zip(caches, cams0):
        r.attach_caches(c, c)
        r.initCacheBlockwise(fvc.raymarch_info(cam, loader.stepsize_info))
    n = sum(W * H for W, H in SIZES)
    res = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    cnt = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    img = torch.zeros((n, 4), dtype=torch.uint8, device="cuda")
    infos1 = [fvc.raymarch_info(c, loader.stepsize_info) for c in cams1]
    r.render_batch_cached(infos1, caches, image=img, results=res, ray_counts=cnt)
    r.synchronize()
    single = []
    for c, cam in zip(caches, cams1):
        r.attach_caches(c, c)
        buf = fvc.RenderBuffer(cam["resolution"])
        r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
        single.append(buf)
    counts = cnt.cpu().numpy()
    assert counts[:, 1].sum() > 0 and counts[:, 0].sum() > 0  # both cache rows and resampled rows
    _check(single, res.cpu().numpy(), counts, img.cpu().numpy())
