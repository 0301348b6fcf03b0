"""MLP precision sweep on the plain tcgen05 path: FP16, BF16, FP8-E4M3.

Each precision renders the same seeded scene; the image (C + T, the white-
background pixel) is compared with the float64 oracle's.  Bounds (measured
values in the comments) are per precision: FP16 keeps the parity bound of the
plain path; BF16 and FP8 are reported as PSNR against the oracle.  The error
behaviour of unsupported combinations is checked too.
"""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import _lib as L
from oracle import oracle as orc
from tests.helpers import psnr, small_camera, tiny_model

pytestmark = pytest.mark.gpu

W, H = 64, 48
BOUNDS = {  # precision: (max-abs bound, PSNR floor in dB); measured on a GB300 in the comments
    fvc.PerformanceRenderer.FP16: (2e-3, 90.0),      # 9.8e-6, 116.5 dB
    fvc.PerformanceRenderer.BF16: (2e-3, 75.0),      # 2.0e-4, 87.4 dB
    fvc.PerformanceRenderer.FP8_E4M3: (2e-2, 55.0),  # 3.4e-3, 64.8 dB
}


@pytest.fixture(scope="module")
def scene():
    d = tiny_model(7, 1)
    loader = fvc.load_data(d)
    cam = small_camera(1001, W, H)
    res, _, _ = orc.OracleModel(d).render_plain(cam)
    return loader, cam, res[..., :3] + res[..., 3:4]


@pytest.mark.parametrize("precision", [0, 1, 2], ids=["fp16", "bf16", "fp8_e4m3"])
def test_precision_against_oracle(scene, precision):
    loader, cam, ref = scene
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.set_precision(precision)
    buf = fvc.RenderBuffer((W, H))
    r.render(fvc.raymarch_info(cam, loader.stepsize_info), buf)
    img = buf.results[..., :3] + buf.results[..., 3:4]
    err = float(np.abs(img - ref).max())
    p = psnr(img, ref)
    print(f"precision {precision}: max-abs {err:.3e} PSNR {p:.1f} dB")
    bound, floor = BOUNDS[precision]
    assert err < bound and p > floor, (err, p)


def test_unsupported_precision_combinations(scene):
    loader, cam, _ = scene
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.set_precision(fvc.PerformanceRenderer.BF16)
    r.set_network_path(False)
    with pytest.raises(L.FvcError) as e:
        r.render(info, fvc.RenderBuffer((W, H)))
    assert "tcgen05" in str(e.value)
    with pytest.raises(L.FvcError):
        r.set_precision(7)
