"""The C++ renderer API (include/fvc.hpp) and the eval program built on it.

CPU: a host-only C++ program checks the reference's type layouts, the
nerfacc camera-file loader, the rigid inverse, CameraInfo::resize and the PNG
writer (decoded here with zlib); eval's argument parsing follows the
reference's (src/eval.cu:88-121: a bad command line prints the usage and
exits 0).  GPU: eval renders a tiny model over a two-frame camera file with
-w -sc and writes the reference's output tree; the cached renders pass the
>= 35 dB check against the plain ones.
"""
import json
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from frustumvolumecaching_gb300 import build as fbuild
from frustumvolumecaching_gb300 import camera as fcam
from tests.helpers import tiny_model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _camera_file(tmp_path, W=40, H=30, n=2):
    cams = [fcam.seeded_camera(1100 + i, width=W, height=H) for i in range(n)]
    p = tmp_path / "transforms.json"
    fcam.write_nerfacc_camera_path(str(p), cams)
    return p, cams


def _read_png(path):
    d = open(path, "rb").read()
    assert d[:8] == b"\x89PNG\r\n\x1a\n"
    off, idat, w, h = 8, b"", 0, 0
    while off < len(d):
        n, = struct.unpack(">I", d[off:off + 4])
        t = d[off + 4:off + 8]
        body = d[off + 8:off + 8 + n]
        crc, = struct.unpack(">I", d[off + 8 + n:off + 12 + n])
        assert zlib.crc32(t + body) & 0xFFFFFFFF == crc
        if t == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
            ch = {6: 4, 0: 1}[body[9]]
        elif t == b"IDAT":
            idat += body
        off += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + ch * w)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, ch) if ch > 1 else rows[:, 1:].reshape(h, w)


def test_cpp_header_host_checks(tmp_path):
    lib = fbuild.build()
    cuda = fbuild.cuda_root()
    exe = tmp_path / "api_check"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "cpp", "api_check.cpp"), "-o", str(exe), "-L", os.path.dirname(lib), "-lfvc",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cam_file, _ = _camera_file(tmp_path)
    png = tmp_path / "check.png"
    r = subprocess.run([str(exe), str(cam_file), str(png)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
    img = _read_png(png)
    expect = (np.arange(7 * 5 * 4) * 37 % 256).astype(np.uint8).reshape(5, 7, 4)
    np.testing.assert_array_equal(img, expect)


def test_eval_bad_command_line_prints_usage():
    exe = fbuild.build_eval()
    r = subprocess.run([exe, "only-one-positional"], capture_output=True, text=True)
    assert r.returncode == 0
    assert "Argument parsing failed!" in r.stdout and "camera-transforms" in r.stdout


@pytest.mark.gpu
def test_eval_writes_reference_output_tree(tmp_path):
    exe = fbuild.build_eval()
    cam_file, cams = _camera_file(tmp_path, W=64, H=48)
    out = tmp_path / "out"
    r = subprocess.run([exe, tiny_model(7, 1), str(cam_file), str(out), "-w", "-sc", "-nrit", "2"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "SANITY CHECK FAILED" not in r.stderr, r.stderr
    for i in range(len(cams)):
        d = out / f"frame_{i:03d}"
        for name in ["no_cache.png", "cache.png", "metrics.json", "timings.json", "rot/5/0.png", "rot/15/300.png",
                     "trans/0.100000.png"]:
            assert (d / name).exists(), name
        assert _read_png(d / "no_cache.png").shape == (48, 64, 4)
        m = json.load(open(d / "metrics.json"))
        assert len(m["rot"]) == 18 and len(m["trans"]) == 6
        assert set(m["rot"][0]) == {"image", "n_bricks_set", "n_bricks_reserved", "overflow", "n_cache_samples", "n_resamples"}
        t = json.load(open(d / "timings.json"))
        assert t["no_cache"]["render_time_ms"] > 0 and len(t["rot"]) == 18


@pytest.mark.gpu
def test_eval_writes_contribution_images(tmp_path):
    """-w -wc: every rotation / translation offset gets <name>_contr_new.png and
    <name>_contr_cache.png, one-channel images of the resampled and cached
    samples' compositing weight; where both are written their sum is the
    pixel's opacity, at most 255 (plus rounding)."""
    exe = fbuild.build_eval()
    cam_file, cams = _camera_file(tmp_path, W=64, H=48)
    out = tmp_path / "out"
    r = subprocess.run([exe, tiny_model(7, 1), str(cam_file), str(out), "-w", "-wc"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    d = out / "frame_000"
    for stem in ["rot/5/0", "rot/10/60", "trans/0.100000"]:
        new = _read_png(d / f"{stem}_contr_new.png")
        cache = _read_png(d / f"{stem}_contr_cache.png")
        assert new.shape == (48, 64) and cache.shape == (48, 64)
        assert (new.astype(int) + cache.astype(int)).max() <= 256
        assert new.any() or cache.any()
