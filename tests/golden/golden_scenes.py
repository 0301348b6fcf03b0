"""Fixed inputs of the marcher golden vectors (shared by make_golden.py and
the tests that replay them against the oracle and the GPU)."""
import math

import numpy as np

R = 128


def occupancy_grid(nlvl: int) -> np.ndarray:
    """uint8 grid, file order l*R^3 + x*R^2 + y*R + z; a cell is occupied when
    an integer hash of (x, y, z, l) is 0 mod 8 (12.5 %), bit-exact anywhere."""
    i = np.arange(R, dtype=np.uint32)
    X, Y, Z = np.meshgrid(i, i, i, indexing="ij")
    out = []
    for l in range(nlvl):
        h = (X * np.uint32(73856093)) ^ (Y * np.uint32(19349663)) ^ (Z * np.uint32(83492791)) ^ np.uint32(l * 1234567)
        h = h ^ (h >> np.uint32(13))
        out.append(((h % np.uint32(8)) == 0).astype(np.uint8).ravel())
    return np.concatenate(out)


def _c2w(eye):
    eye = np.asarray(eye, np.float64)
    fwd = -eye / np.linalg.norm(eye)
    up = np.array([0.0, 0.0, 1.0])
    right = np.cross(fwd, up); right /= np.linalg.norm(right)
    down = np.cross(fwd, right)
    m = np.zeros((3, 4), np.float32)
    m[:, 0], m[:, 1], m[:, 2], m[:, 3] = right, down, fwd, eye
    return m.ravel()


def _f(h, fov=50.0):
    return float(np.float32(0.5 * h / math.tan(math.radians(fov) * 0.5)))


SCENES = {
    "c1": dict(nlvl=1, contraction=0, aabb=[-1.5, -1.5, -1.5, 1.5, 1.5, 1.5], caabb=[-1.5, -1.5, -1.5, 1.5, 1.5, 1.5],
               cone=0.0, stepsize=3.0 / 1024.0, near=0.0, far=1e10, W=256, H=256, fx=_f(256), fy=_f(256), px=128.0,
               py=128.0, c2w=_c2w([2.31, -2.72, 1.9]), max_steps=4096, pix_stride=16, seed=11),
    "c2": dict(nlvl=3, contraction=1, aabb=[-6.0, -6.0, -6.0, 6.0, 6.0, 6.0], caabb=[-1.5, -1.5, -1.5, 1.5, 1.5, 1.5],
               cone=1.0 / 256.0, stepsize=math.sqrt(3.0) / 1024.0, near=0.0, far=1e10, W=1920, H=1080, fx=_f(1080),
               fy=_f(1080), px=960.0, py=540.0, c2w=_c2w([-3.1, 2.2, 1.2]), max_steps=8192, pix_stride=120, seed=12),
}


def pixels(sc) -> np.ndarray:
    s = sc["pix_stride"]
    xs = np.arange(s // 2, sc["W"], s)
    ys = np.arange(s // 3, sc["H"], max(1, s * sc["H"] // sc["W"]))
    P = np.stack(np.meshgrid(xs, ys, indexing="xy"), -1).reshape(-1, 2)
    return P[:256].astype(np.int32)


def points(sc) -> np.ndarray:
    rng = np.random.default_rng(sc["seed"])
    a = np.asarray(sc["aabb"], np.float64)
    return rng.uniform(a[:3], a[3:], size=(256, 3)).astype(np.float32)
