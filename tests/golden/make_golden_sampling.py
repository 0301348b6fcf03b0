"""Regenerates tests/golden/sampling.npz from the reference's own sampling
code of non-deterministic ray generation (include/util/random_val.h,
include/util/quat.h, generateRay in include/raymarch_common.h), compiled on
the host by oracle/Makefile (target ``ref``) into oracle/_ref/ref_sampling.

Run from the repository root where the reference tree is available:
    make -C oracle ref REF=<reference checkout>
    python tests/golden/make_golden_sampling.py

Inputs are seeded; the npz holds them with the reference's outputs.
"""
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from frustumvolumecaching_gb300 import camera as fcam  # noqa: E402


def rotation(q):
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def inputs():
    rng = np.random.default_rng(2024)
    sob = np.stack([rng.integers(0, 2 ** 32, 400, dtype=np.uint64), np.tile(np.arange(5), 80)], 1).astype(np.uint32)
    sob[:32, 0] = 1 << np.arange(32, dtype=np.uint64)  # every direction number on its own
    ld = rng.integers(0, 2 ** 32, (200, 2), dtype=np.uint64).astype(np.uint32)
    spp = np.arange(256, dtype=np.uint32)
    toff = np.stack([rng.integers(0, 64, 200), rng.integers(0, 1920 * 1080, 200)], 1).astype(np.uint32)
    disk = rng.uniform(-1, 1, (400, 2)).astype(np.float32)
    disk[:4] = [[0.5, 0.5], [-0.25, 0.75], [1.0, -1.0], [0.0, 0.3]]
    sl = []
    for k in range(100):
        a = np.concatenate([rotation(rng.normal(size=4)), rng.uniform(-3, 3, (3, 1))], 1)
        if k % 3 == 0:   # a small turn, as consecutive frames of a camera path
            b = np.concatenate([a[:, :3] @ rotation(np.array([1.0, *rng.normal(scale=0.01, size=3)])),
                                a[:, 3:] + rng.normal(scale=0.05, size=(3, 1))], 1)
        else:
            b = np.concatenate([rotation(rng.normal(size=4)), rng.uniform(-3, 3, (3, 1))], 1)
        sl.append(np.concatenate([a.ravel(), b.ravel(), [rng.uniform(0, 1)]]))
    sl = np.asarray(sl, np.float32)
    cam = fcam.seeded_camera(77, width=320, height=240)
    c2w = np.asarray(cam["cam2world"], np.float64)
    nxt = fcam.seeded_camera(78, width=320, height=240)["cam2world"]
    rays = np.stack([rng.integers(0, 320, 300), rng.integers(0, 240, 300), rng.integers(0, 16, 300),
                     np.tile(np.arange(4), 75)], 1).astype(np.int32)
    return dict(sobol_in=sob, ld_in=ld, spp_in=spp, toff_in=toff, disk_in=disk, slerp_in=sl, rays_in=rays,
                cam_res=np.array([320, 240], np.int32), cam_intr=np.asarray([*cam["focal"], *cam["principal"]], np.float32),
                cam_c2w=c2w.astype(np.float32), cam_next=np.asarray(nxt, np.float32),
                cam_lens=np.array([0.05, 3.5], np.float32),
                scene=np.array([-1.5, -1.5, -1.5, 1.5, 1.5, 1.5, 1.0 / 256.0, 3.0 / 1024.0, 0.0, 1e10], np.float32),
                scene_nlvl=np.int32(1))


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_sampling")
    if not os.path.exists(exe):
        raise SystemExit("build oracle/_ref/ref_sampling first (make -C oracle ref)")
    d = inputs()
    inp, outp = "/tmp/fvc_sampling.in", "/tmp/fvc_sampling.out"
    with open(inp, "wb") as f:
        for key in ("sobol_in", "ld_in"):
            f.write(struct.pack("<i", d[key].shape[0])); f.write(d[key].astype("<u4").tobytes())
        f.write(struct.pack("<i", d["spp_in"].size)); f.write(d["spp_in"].astype("<u4").tobytes())
        f.write(struct.pack("<i", d["toff_in"].shape[0])); f.write(d["toff_in"].astype("<u4").tobytes())
        f.write(struct.pack("<i", d["disk_in"].shape[0])); f.write(d["disk_in"].astype("<f4").tobytes())
        f.write(struct.pack("<i", d["slerp_in"].shape[0])); f.write(d["slerp_in"].astype("<f4").tobytes())
        f.write(d["cam_res"].astype("<i4").tobytes()); f.write(d["cam_intr"].astype("<f4").tobytes())
        f.write(d["cam_c2w"].astype("<f4").tobytes()); f.write(d["cam_next"].astype("<f4").tobytes())
        f.write(d["cam_lens"].astype("<f4").tobytes())
        f.write(d["scene"].astype("<f4").tobytes()); f.write(struct.pack("<i", int(d["scene_nlvl"])))
        f.write(struct.pack("<i", d["rays_in"].shape[0])); f.write(d["rays_in"].astype("<i4").tobytes())
    subprocess.run([exe, inp, outp], check=True)
    b = open(outp, "rb").read()
    o = 0

    def take(dtype, n):
        nonlocal o
        a = np.frombuffer(b, dtype, n, o)
        o += a.nbytes
        return a.copy()

    d["sobol_out"] = take("<u4", d["sobol_in"].shape[0])
    ld = take("<f4", 3 * d["ld_in"].shape[0]).reshape(-1, 3)
    d["ld_out"], d["ld2_out"] = ld[:, 0], ld[:, 1:]
    d["spp_out"] = take("<f4", 2 * d["spp_in"].size).reshape(-1, 2)
    d["toff_out"] = take("<f4", d["toff_in"].shape[0])
    d["disk_out"] = take("<f4", 2 * d["disk_in"].shape[0]).reshape(-1, 2)
    d["slerp_out"] = take("<f4", 12 * d["slerp_in"].shape[0]).reshape(-1, 12)
    d["rays_out"] = take("<f4", 8 * d["rays_in"].shape[0]).reshape(-1, 8)
    assert o == len(b), (o, len(b))
    np.savez_compressed(os.path.join(HERE, "sampling.npz"), **d)
    print("sampling golden:", {k: v.shape for k, v in d.items() if k.endswith("_out")})


if __name__ == "__main__":
    main()
