"""The headless camera-path renderer (render_path, the viewer's
renderCameraPath) end to end: every frame written; frame 0 of the plain run
equals a render of the same spline cameras through the Python API (motion
blur toward the next frame's pose, spp jittered samples accumulated in the
progressive image) byte for byte; the cached run rebuilds at frame 0 and
then only when the cache-update rule asks."""
import json
import subprocess
import zlib

import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import build as fbuild
from tests.helpers import tiny_model
from tests.test_camera_path import make_path, run_eval, write_path

pytestmark = pytest.mark.gpu

W, H, SPP, FPS, DUR = 64, 48, 2, 4.0, 1.0
SETTINGS = {"resolution": [W, H], "fov_x": 50.0, "render_from_cache": False, "auto_cache_update": False,
            "cache_update_distance": 0.05, "cache_min_hit_ratio": 0.5, "spp": SPP, "fps": FPS, "duration": DUR,
            "shutter_fraction": 0.5, "quality": 10}


def read_png(path):
    """RGBA8 PNG of unfiltered rows (render_path's writer)"""
    b = open(path, "rb").read()
    o, idat, w, h = 8, b"", 0, 0
    while o < len(b):
        n = int.from_bytes(b[o:o + 4], "big")
        kind = b[o + 4:o + 8]
        data = b[o + 8:o + 8 + n]
        if kind == b"IHDR":
            w, h = int.from_bytes(data[:4], "big"), int.from_bytes(data[4:8], "big")
        elif kind == b"IDAT":
            idat += data
        o += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    assert not raw[:, 0].any()
    return raw[:, 1:].reshape(h, w, 4)


def _run(tmp_path, name, extra):
    d = tiny_model(7, 1)
    keys = make_path(np.random.default_rng(9), n=3)
    write_path(tmp_path / "path.json", keys, SETTINGS)
    out = tmp_path / name
    exe = fbuild.build_render_path()
    subprocess.run([exe, d, str(tmp_path / "path.json"), str(out), *extra], check=True, capture_output=True, text=True)
    frames = json.load(open(out / "frames.json"))
    return d, out, frames


def test_plain_path_frames_match_python_renders(tmp_path):
    d, out, frames = _run(tmp_path, "plain", [])
    n = int(FPS * DUR)
    assert [f["frame"] for f in frames] == list(range(n)) and not any(f["cache_update"] for f in frames)
    loader = fvc.load_data(d)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    for i in (0, n - 1):
        cams = run_eval(tmp_path / "path.json", i / n, (i + 1) / n, 2)
        cur, nxt = cams
        fx = (W * 0.5) / np.tan(np.radians(50.0) * 0.5)
        c2w = np.asarray(cur["cam2world"], np.float32)
        cam = {"resolution": (W, H), "is_open_gl": False, "focal": (np.float32(fx), np.float32(fx)),
               "principal": (W * 0.5, H * 0.5), "cam2world": c2w, "deterministic": False, "motion_blur": True,
               "next_cam2world": np.asarray(nxt["cam2world"], np.float32),
               "aperature": cur["aperture_size"], "focus_z": cur["focus_distance"]}
        buf = fvc.RenderBuffer((W, H))
        for s in range(SPP):
            r.render(fvc.raymarch_info(dict(cam, sample_index=s), loader.stepsize_info), buf)
        png = read_png(out / f"frame_{i:06d}.png")
        # the camera of the spline printed with 9 digits may differ from the program's in the last bit
        diff = np.abs(png.astype(np.int32) - buf.image.astype(np.int32))
        print(f"\nframe {i}: pixels off {(diff > 0).mean():.4f}, max {diff.max()}")
        assert (diff > 1).mean() < 0.01 and (diff > 0).mean() < 0.05


def test_cached_path_follows_the_cache_update_rule(tmp_path):
    _, out, frames = _run(tmp_path, "cached", ["-cache", "-auto", "-frames", "6"])
    assert len(frames) == 6 and frames[0]["cache_update"]
    for prev, f in zip(frames, frames[1:]):
        if not f["cache_update"]:
            assert prev["hit_ratio"] >= SETTINGS["cache_min_hit_ratio"]
    assert any(f["hit_ratio"] > 0 for f in frames)
    for f in frames:
        assert read_png(out / f"frame_{f['frame']:06d}.png").shape == (H, W, 4)
