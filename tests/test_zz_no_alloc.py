"""The allocation-free render entry point (fvc_render_noalloc).

It is for callers that cannot allocate GPU memory while they render; its
scratch is a file-scope device array inside libfvc.so.  This file is
collected last so a failure here leaves the rest of the suite already run.
The test calls the entry point through the C ABI twice in a row and checks
both results against the allocating render path (fvc_render), and that an
image beyond the array's stated maximum is refused.  During the two calls the
library's allocation hook is armed to fail the very next device allocation
(fvc_debug_fail_allocation(0)), so a call that allocated anything through the
library would fail instead of returning FVC_OK.
"""
import ctypes as C

import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import _lib as L
from tests.helpers import small_camera, tiny_model

pytestmark = pytest.mark.gpu

COLOR_ATOL = 2e-3  # the pixel tolerance of the parity tests


def _device_outputs(torch, W, H):
    img = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    res = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    cnt = torch.zeros((H, W, 4), dtype=torch.int32, device="cuda")
    out = L.RenderOutputs()
    out.image_rgba8, out.results, out.ray_counts = img.data_ptr(), res.data_ptr(), cnt.data_ptr()
    return out, img, res, cnt


def test_noalloc_render_matches_allocating_render_twice():
    torch = pytest.importorskip("torch")
    loader = fvc.load_data(tiny_model(7, 1))
    W, H = 64, 48
    cam = small_camera(1001, W, H)
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    ref = fvc.RenderBuffer((W, H))
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.render(info, ref)
    lib = L.load()
    outs = [_device_outputs(torch, W, H) for _ in range(2)]  # torch allocates these before the hook is armed
    torch.cuda.synchronize()
    try:
        assert lib.fvc_debug_fail_allocation(0) == 0  # the library's next device allocation fails
        for out, *_ in outs:
            rc = lib.fvc_render_noalloc(loader.nerf_network.handle, C.byref(info), C.byref(out), None)
            assert rc == 0, lib.fvc_last_error().decode()
    finally:
        lib.fvc_debug_fail_allocation(-1)
    torch.cuda.synchronize()
    for call, (out, img, res, cnt) in enumerate(outs):
        got = res.cpu().numpy()
        assert np.abs(got - ref.results).max() <= COLOR_ATOL, call
        np.testing.assert_array_equal(cnt.cpu().numpy(), ref.ray_counts)
        np.testing.assert_array_equal(img.cpu().numpy(), ref.image)


def test_noalloc_render_rejects_images_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    loader = fvc.load_data(tiny_model(7, 1))
    W, H = 512, 256  # 131072 rays > FVC_NOALLOC_MAX_RAYS (65536)
    cam = small_camera(1001, W, H)
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    out, *_ = _device_outputs(torch, W, H)
    lib = L.load()
    rc = lib.fvc_render_noalloc(loader.nerf_network.handle, C.byref(info), C.byref(out), None)
    assert rc == 6
    assert "65536" in lib.fvc_last_error().decode()
