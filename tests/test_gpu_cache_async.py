"""The double-buffered cache update of the reference's viewer
(realtime_viewer/src/application.cu:168-184 with CacheRenderer's
_low_priority_stream, src/cache_renderer.cu:819-825,931-1051): one thread
builds the next cache while another keeps rendering from the current one,
then the caches swap.  The build runs on the renderer's lowest-priority
stream under the write lock, the renders on the renderer's stream under the
read lock, so the two proceed together; the frame rendered after the swap is
the frame of the synchronous sequence, bit for bit."""
import threading

import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from tests.helpers import small_camera, tiny_model

pytestmark = pytest.mark.gpu


def _rotated(cam0, W, H, deg):
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(deg)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    return fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)


def _renderer(loader, W, H):
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings())
    return r, (c0, c1)


def test_build_in_a_second_thread_while_rendering():
    loader = fvc.load_data(tiny_model(7, 1))
    W, H = 96, 64
    cam0 = small_camera(1001, W, H)
    cam1 = _rotated(cam0, W, H, 2.0)
    info0 = fvc.raymarch_info(cam0, loader.stepsize_info)
    info1 = fvc.raymarch_info(cam1, loader.stepsize_info)

    # synchronous sequence: build at view 0, swap, build at view 1, swap, render view 1
    ref_r, _ = _renderer(loader, W, H)
    ref_r.initCacheBlockwise(info0)
    ref_r.swapCache()
    ref_r.initCacheBlockwise(info1)
    ref_r.swapCache()
    ref = fvc.RenderBuffer((W, H))
    ref_r.render(info1, ref)

    # double-buffered: the view-1 build runs in a worker thread while the main
    # thread renders view 0 from the view-0 cache
    r, _ = _renderer(loader, W, H)
    r.initCacheBlockwise(info0)
    r.swapCache()
    first = fvc.RenderBuffer((W, H))
    r.render(info0, first)
    errors = []

    def build():
        try:
            r.initCacheBlockwise(info1)
        except Exception as e:  # reported by the main thread
            errors.append(e)

    worker = threading.Thread(target=build)
    worker.start()
    frames = 0
    buf = fvc.RenderBuffer((W, H))
    while worker.is_alive() or frames < 2:
        r.render(info0, buf)
        np.testing.assert_array_equal(buf.results, first.results)  # the current cache is untouched by the build
        frames += 1
    worker.join(timeout=300)
    assert not worker.is_alive() and not errors, errors
    r.swapCache()
    out = fvc.RenderBuffer((W, H))
    r.render(info1, out)
    np.testing.assert_array_equal(out.results, ref.results)
    np.testing.assert_array_equal(out.ray_counts, ref.ray_counts)
    assert r._render_stats.n_cache_hits == ref_r._render_stats.n_cache_hits > 0
