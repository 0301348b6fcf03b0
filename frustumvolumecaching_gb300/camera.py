"""Cameras and camera paths for the synthetic workloads.

Camera convention is the reference's non-OpenGL one (``is_open_gl = false``):
camera space x right, y down, z forward, ``cam2world = [right | down |
forward | eye]`` as a 3x4 row-major matrix (CameraMatrix,
include/common.h:22-62; generateRayDir, include/raymarch_common.h:190-201).
``world2cam`` is ``CameraMatrix::inverse`` (transpose of the rotation and
``-R^T t``), evaluated in float32 in the same operation order.
"""
from __future__ import annotations

import math

import numpy as np


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 0.0, 1.0)) -> np.ndarray:
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    upv = np.asarray(up, np.float64)
    if abs(np.dot(fwd, upv)) > 0.999:
        upv = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, upv)
    right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    m = np.zeros((3, 4), np.float32)
    m[:, 0], m[:, 1], m[:, 2], m[:, 3] = right, down, fwd, eye
    return m


def inverse(c2w: np.ndarray) -> np.ndarray:
    """CameraMatrix::inverse (include/common.h:44-55) in float32 with the
    reference's left-to-right dot product."""
    c2w = np.asarray(c2w, np.float32)
    out = np.zeros((3, 4), np.float32)
    t = c2w[:, 3]
    for r in range(3):
        rot = c2w[:, r]  # column r of R == row r of R^T
        out[r, :3] = rot
        d = np.float32(np.float32(rot[0] * t[0]) + np.float32(rot[1] * t[1]))
        d = np.float32(d + np.float32(rot[2] * t[2]))
        out[r, 3] = -d
    return out


def sphere_position(rng: np.random.Generator, radius: float) -> np.ndarray:
    v = rng.normal(size=3)
    v /= np.linalg.norm(v)
    return v * radius


def focal_from_fov(height: int, fov_deg: float) -> float:
    return 0.5 * height / math.tan(math.radians(fov_deg) * 0.5)


def camera_dict(c2w: np.ndarray, width: int, height: int, fov_deg: float = 50.0) -> dict:
    """Fields of CameraInfo (include/common.h:166-195)."""
    f = np.float32(focal_from_fov(height, fov_deg))
    return {
        "resolution": (width, height), "is_open_gl": False,
        "focal": (float(f), float(f)), "principal": (width * 0.5, height * 0.5),
        "cam2world": np.asarray(c2w, np.float32), "world2cam": inverse(c2w),
    }


def seeded_camera(seed: int, radius: float = 4.0, width: int = 256, height: int = 256, fov_deg: float = 50.0) -> dict:
    """One camera on a radius-``radius`` sphere looking at the origin; the
    position comes from the camera stream of the workload seed."""
    rng = np.random.default_rng([seed, 1])
    return camera_dict(look_at(sphere_position(rng, radius)), width, height, fov_deg)


def rotation_path(seed: int, n_frames: int = 60, deg_per_frame: float = 0.5, step_per_frame: float = 0.01,
                  radius: float = 4.0, width: int = 1920, height: int = 1080, fov_deg: float = 50.0) -> list[dict]:
    """Camera path of the cached workload: orbit ``deg_per_frame`` per frame
    about the world up axis (z) through the origin while moving
    ``step_per_frame`` units per frame towards the origin, always looking at
    the origin."""
    rng = np.random.default_rng([seed, 1])
    eye0 = sphere_position(rng, radius)
    cams = []
    for i in range(n_frames):
        a = math.radians(deg_per_frame * i)
        rot = np.array([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])
        e = rot @ eye0
        e = e * (np.linalg.norm(e) - step_per_frame * i) / np.linalg.norm(e)
        cams.append(camera_dict(look_at(e), width, height, fov_deg))
    return cams


def write_nerfacc_camera_path(path: str, cams: list[dict], image_stem: str = "frame") -> None:
    """The cameras as a nerfacc camera file (the format load_camerapath reads,
    src/loader.cu:322-343 with include/parse_helper.h:66-107): width, height,
    is_open_gl, 3x3 intrinsics and frames of 4x4 cam2world rows + image_path."""
    import json

    c0 = cams[0]
    W, H = c0["resolution"]
    (fx, fy), (cx, cy) = c0["focal"], c0["principal"]
    frames = []
    for i, c in enumerate(cams):
        m = np.asarray(c["cam2world"], np.float64)
        rows = [[float(v) for v in m[r]] for r in range(3)] + [[0.0, 0.0, 0.0, 1.0]]
        frames.append({"transform_matrix": rows, "image_path": f"{image_stem}_{i:03d}"})
    doc = {"width": int(W), "height": int(H), "is_open_gl": bool(c0["is_open_gl"]),
           "intrinsics": [[float(fx), 0.0, float(cx)], [0.0, float(fy), float(cy)], [0.0, 0.0, 1.0]], "frames": frames}
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)
