"""Regenerates the golden vectors in this directory from the reference's own
marcher math (include/raymarch_common.h, include/common.h), compiled on the
host by oracle/Makefile (target ``ref``) into oracle/_ref/ref_golden.

Run from the repository root where the reference tree is available:
    make -C oracle ref REF=<reference checkout>
    python tests/golden/make_golden.py

The scenes use an occupancy grid defined by an integer hash of the cell
coordinates (bit-exact on every platform), fixed cameras and seeded points.
"""
import os
import struct
import subprocess
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden.golden_scenes import SCENES, occupancy_grid, pixels, points  # noqa: E402


def write_input(path, sc):
    grid = occupancy_grid(sc["nlvl"])
    pix = pixels(sc)
    pts = points(sc)
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", sc["nlvl"], sc["contraction"]))
        f.write(np.asarray(sc["aabb"] + sc["caabb"], np.float32).tobytes())
        f.write(np.asarray([sc["cone"], sc["stepsize"], sc["near"], sc["far"]], np.float32).tobytes())
        f.write(struct.pack("<ii", sc["W"], sc["H"]))
        f.write(np.asarray([sc["fx"], sc["fy"], sc["px"], sc["py"]], np.float32).tobytes())
        f.write(np.asarray(sc["c2w"], np.float32).tobytes())
        f.write(struct.pack("<i", pix.shape[0]))
        f.write(pix.astype(np.int32).tobytes())
        f.write(struct.pack("<i", sc["max_steps"]))
        f.write(struct.pack("<i", pts.shape[0]))
        f.write(pts.astype(np.float32).tobytes())
        f.write(grid.tobytes())
    return pix.shape[0], pts.shape[0]


def parse_output(path, n_pix, n_pts):
    b = open(path, "rb").read()
    o = 0

    def take(fmt):
        nonlocal o
        v = struct.unpack_from(fmt, b, o)
        o += struct.calcsize(fmt)
        return v

    out = {}
    out["steps"] = np.asarray(take("<8f"), np.float32)  # dt_min dt_max t_min t_max i_min i_max log1p_c near_i
    out["world2cam"] = np.asarray(take("<12f"), np.float32)
    out["max_step"] = np.float32(take("<f")[0])
    hits, start, far, org, dr, nsteps, crc, occ_steps, occ_t0, occ_off = [], [], [], [], [], [], [], [], [], [0]
    for _ in range(n_pix):
        h, s, fa = take("<iff")
        og = take("<3f")
        d = take("<3f")
        n, = take("<i")
        t0 = np.frombuffer(b, np.float32, n, o)
        o += 4 * n
        oc = np.frombuffer(b, np.uint8, n, o)
        o += n
        hits.append(h); start.append(s); far.append(fa); org.append(og); dr.append(d); nsteps.append(n)
        crc.append(zlib.crc32(t0.tobytes()) ^ (zlib.crc32(oc.tobytes()) << 1 & 0xFFFFFFFF))
        idx = np.nonzero(oc)[0]
        occ_steps.append(idx.astype(np.int32)); occ_t0.append(t0[idx]); occ_off.append(occ_off[-1] + idx.size)
    out.update(hits=np.asarray(hits, np.int32), start=np.asarray(start, np.float32), far=np.asarray(far, np.float32),
               origin=np.asarray(org, np.float32), dir=np.asarray(dr, np.float32), n_steps=np.asarray(nsteps, np.int32),
               crc=np.asarray(crc, np.uint64), occ_steps=np.concatenate(occ_steps), occ_t0=np.concatenate(occ_t0),
               occ_off=np.asarray(occ_off, np.int64))
    pt = []
    for _ in range(n_pts):
        pt.append(take("<ff3fi3ff"))
    pt = np.asarray(pt, np.float64)
    out["pt_step_from_t"] = pt[:, 0].astype(np.float32)
    out["pt_t_from_step"] = pt[:, 1].astype(np.float32)
    out["pt_contract"] = pt[:, 2:5].astype(np.float32)
    out["pt_occ"] = pt[:, 5].astype(np.int32)
    out["pt_froxel"] = pt[:, 6:9].astype(np.float32)
    out["pt_froxel_t"] = pt[:, 9].astype(np.float32)
    ints = [take("<Ii3i") for _ in range(64)]
    out["morton"] = np.asarray([v[0] for v in ints], np.uint32)
    out["pack3d"] = np.asarray([v[1] for v in ints], np.int32)
    out["to3d"] = np.asarray([v[2:5] for v in ints], np.int32)
    assert o == len(b), (o, len(b))
    return out


def main():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_golden")
    if not os.path.exists(exe):
        raise SystemExit("build oracle/_ref/ref_golden first (make -C oracle ref)")
    for name, sc in SCENES.items():
        inp = os.path.join("/tmp", f"fvc_golden_{name}.in")
        outp = os.path.join("/tmp", f"fvc_golden_{name}.out")
        n_pix, n_pts = write_input(inp, sc)
        subprocess.run([exe, inp, outp], check=True)
        res = parse_output(outp, n_pix, n_pts)
        np.savez_compressed(os.path.join(HERE, f"march_{name}.npz"), **res)
        print(name, "rays", n_pix, "steps", int(res["n_steps"].sum()), "occupied", int(res["occ_off"][-1]))


if __name__ == "__main__":
    main()
