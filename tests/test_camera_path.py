"""The viewer's key-framed camera path (include/fvc_camera_path.hpp, the
spline of realtime_viewer/src/camera_path.cu:14-48 and eval_camera_path of
realtime_viewer/include/camera_path.h:91-99) through render_path's -eval
mode, against a float64 restatement of the same construction: Catmull-Rom as
three levels of key-frame lerps, slerp on the short arc for the rotation,
linear for translation, aperture and focus; the end key frames repeated."""
import json
import os
import subprocess

import numpy as np
import pytest

from frustumvolumecaching_gb300 import build as fbuild


def _quat_of(R):
    """unit quaternion (w, x, y, z) of a rotation matrix"""
    w = np.sqrt(max(0.0, 1.0 + R[0, 0] + R[1, 1] + R[2, 2])) / 2.0
    x = np.copysign(np.sqrt(max(0.0, 1.0 + R[0, 0] - R[1, 1] - R[2, 2])) / 2.0, R[2, 1] - R[1, 2])
    y = np.copysign(np.sqrt(max(0.0, 1.0 - R[0, 0] + R[1, 1] - R[2, 2])) / 2.0, R[0, 2] - R[2, 0])
    z = np.copysign(np.sqrt(max(0.0, 1.0 - R[0, 0] - R[1, 1] + R[2, 2])) / 2.0, R[1, 0] - R[0, 1])
    q = np.array([w, x, y, z])
    return q / np.linalg.norm(q)


def _rot(q):
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _slerp(a, b, t):
    ct = float(a @ b)
    if ct < 0:
        b, ct = -b, -ct
    if ct > 1 - 2 ** -23:
        return a * (1 - t) + b * t
    ang = np.arccos(ct)
    return (np.sin((1 - t) * ang) * a + np.sin(t * ang) * b) / np.sin(ang)


def _lerp(p0, p1, t, t0, t1):
    t = (t - t0) / (t1 - t0)
    R1 = p1["R"] if p1["R"] @ p0["R"] >= 0 else -p1["R"]
    R = _slerp(p0["R"], R1, t)
    return {"R": R / np.linalg.norm(R), "T": p0["T"] + (p1["T"] - p0["T"]) * t,
            "a": p0["a"] + (p1["a"] - p0["a"]) * t, "f": p0["f"] + (p1["f"] - p0["f"]) * t}


def _spline(t, p0, p1, p2, p3):
    q0, q1, q2 = _lerp(p0, p1, t, -1, 0), _lerp(p1, p2, t, 0, 1), _lerp(p2, p3, t, 1, 2)
    return _lerp(_lerp(q0, q1, t, -1, 1), _lerp(q1, q2, t, 0, 2), t, 0, 1)


def _eval(keys, t):
    t *= len(keys) - 1
    i = int(np.floor(t))
    k = lambda j: keys[min(max(j, 0), len(keys) - 1)]  # noqa: E731
    return _spline(t - np.floor(t), k(i - 1), k(i), k(i + 1), k(i + 2))


def make_path(rng, n=4):
    keys = []
    for i in range(n):
        eye = np.array([4 * np.cos(0.4 * i), 4 * np.sin(0.4 * i), 1.0 + 0.2 * i])
        f = -eye / np.linalg.norm(eye)
        r = np.cross(f, [0, 0, 1.0]); r /= np.linalg.norm(r)
        u = np.cross(f, r)
        R = np.stack([r, u, f], 1)
        keys.append({"R": _quat_of(R), "T": eye + rng.normal(scale=0.05, size=3), "a": 0.01 * i, "f": 3.0 + 0.1 * i})
    return keys


def write_path(path, keys, settings=None):
    doc = {"path": [{"R": [float(k["R"][1]), float(k["R"][2]), float(k["R"][3]), float(k["R"][0])],
                     "T": [float(v) for v in k["T"]], "aperture_size": float(k["a"]), "focus_distance": float(k["f"])}
                    for k in keys]}
    if settings:
        doc["settings"] = settings
    with open(path, "w") as f:
        json.dump(doc, f)


def run_eval(path_file, t0, t1, n):
    exe = fbuild.build_render_path()
    out = subprocess.run([exe, str(path_file), "-eval", str(t0), str(t1), str(n)], check=True, capture_output=True, text=True)
    return [json.loads(line) for line in out.stdout.splitlines() if line.strip()]


def test_spline_against_float64_restatement(tmp_path):
    keys = make_path(np.random.default_rng(3))
    write_path(tmp_path / "p.json", keys)
    got = run_eval(tmp_path / "p.json", 0.0, 1.0, 37)
    worst = 0.0
    for g in got:
        ref = _eval(keys, g["t"])
        m = np.asarray(g["cam2world"])
        worst = max(worst, float(np.abs(m[:, :3] - _rot(ref["R"])).max()), float(np.abs(m[:, 3] - ref["T"]).max()))
        assert abs(g["aperture_size"] - ref["a"]) < 1e-6 and abs(g["focus_distance"] - ref["f"]) < 1e-5
    assert worst < 2e-5, worst


def test_spline_passes_through_key_frames_and_clamps_ends(tmp_path):
    keys = make_path(np.random.default_rng(4), n=5)
    write_path(tmp_path / "p.json", keys)
    got = run_eval(tmp_path / "p.json", 0.0, 1.0, 5)  # t = k / 4: key frame k
    for k, g in zip(keys, got):
        m = np.asarray(g["cam2world"])
        np.testing.assert_allclose(m[:, :3], _rot(k["R"]), atol=2e-6)
        np.testing.assert_allclose(m[:, 3], k["T"], atol=2e-6)
        np.testing.assert_allclose(np.linalg.norm(g["R"]), 1.0, atol=1e-6)


def test_single_key_frame_is_constant(tmp_path):
    keys = make_path(np.random.default_rng(5), n=1)
    write_path(tmp_path / "p.json", keys)
    got = run_eval(tmp_path / "p.json", 0.0, 0.99, 4)
    for g in got:
        np.testing.assert_allclose(np.asarray(g["cam2world"])[:, 3], keys[0]["T"], atol=1e-6)


@pytest.mark.parametrize("bad", ["missing.json"])
def test_missing_path_file_fails(tmp_path, bad):
    exe = fbuild.build_render_path()
    r = subprocess.run([exe, str(tmp_path / bad), "-eval", "0", "1", "2"], capture_output=True, text=True)
    assert r.returncode != 0
    assert os.path.exists(exe)
