"""Device golden vectors of the marcher: the reference's marcher math compiled
for the GPU with the reference's own flags (oracle/ref_golden_dev.cu, built
by oracle/Makefile into oracle/_ref/ref_golden_dev.cubin with -use_fast_math).

Two steps, on two machines:

  prep (where the reference tree is available; no GPU needed)
      make -C oracle ref REF=<reference checkout>
      python tests/golden/make_golden_dev.py prep
    runs oracle/_ref/ref_golden on each golden scene, which writes the
    RaymarchInfo / SceneInfo structs as the reference's host code fills them
    (StepsizeInfo::setAdditionalInfo, CameraMatrix::inverse) and the Morton
    occupancy bitfield, then widens the pixel list to a dense grid over the
    frame plus the scene's 256 golden pixels: oracle/_ref/golden_dev_<scene>.bin.

  run (on a GPU; needs oracle/_ref from the prep step and torch)
      python tests/golden/make_golden_dev.py run <out_dir>
    loads the cubin through the CUDA driver API, marches every pixel and
    writes <out_dir>/march_<scene>_dev.npz; copy those into tests/golden/.

npz keys: stride (dense grid step in pixels, starting at pixel (0, 0)),
hits / steps / occupied [H/stride, W/stride] (steps and occupied are counts
over the whole ray), and for the scene's golden pixels (golden_scenes.pixels)
g_hits, g_steps, g_occupied and g_t0_hash (FNV-1a over the bytes of each
occupied step's t0, low byte first).
"""
import ctypes as C
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden.golden_scenes import SCENES, pixels  # noqa: E402
from tests.golden.make_golden import write_input  # noqa: E402

REF_DIR = os.path.join(ROOT, "oracle", "_ref")
STRIDE = {"c1": 1, "c2": 4}


def dense_pixels(sc, stride):
    xs = np.arange(0, sc["W"], stride, dtype=np.int32)
    ys = np.arange(0, sc["H"], stride, dtype=np.int32)
    return np.stack(np.meshgrid(xs, ys, indexing="xy"), -1).reshape(-1, 2)


def prep():
    exe = os.path.join(REF_DIR, "ref_golden")
    if not os.path.exists(exe):
        raise SystemExit("build oracle/_ref/ref_golden first (make -C oracle ref)")
    for name, sc in SCENES.items():
        inp = os.path.join("/tmp", f"fvc_golden_{name}.in")
        outp = os.path.join("/tmp", f"fvc_golden_{name}.out")
        devp = os.path.join("/tmp", f"fvc_golden_{name}.dev")
        write_input(inp, sc)
        subprocess.run([exe, inp, outp, devp], check=True)
        b = open(devp, "rb").read()
        srm, ssi = struct.unpack_from("<ii", b, 0)
        o = 8
        structs = b[o:o + srm + ssi]
        o += srm + ssi
        n_pix, = struct.unpack_from("<i", b, o)
        o += 4 + 8 * n_pix
        max_steps, nlvl, nb = struct.unpack_from("<iii", b, o)
        o += 12
        bits = b[o:o + nb]
        assert o + nb == len(b)
        pix = np.concatenate([dense_pixels(sc, STRIDE[name]), pixels(sc)]).astype(np.int32)
        with open(os.path.join(REF_DIR, f"golden_dev_{name}.bin"), "wb") as f:
            f.write(struct.pack("<ii", srm, ssi))
            f.write(structs)
            f.write(struct.pack("<i", pix.shape[0]))
            f.write(pix.tobytes())
            f.write(struct.pack("<iii", max_steps, nlvl, nb))
            f.write(bits)
        print(name, "device input", pix.shape[0], "pixels")


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with CUresult {rc}")


def run(out_dir):
    import torch

    cubin = open(os.path.join(REF_DIR, "ref_golden_dev.cubin"), "rb").read()
    torch.zeros(1, device="cuda")  # makes the primary context current on this thread
    cu = C.CDLL("libcuda.so.1")
    mod, fn = C.c_void_p(), C.c_void_p()
    _check(cu.cuModuleLoadData(C.byref(mod), C.c_char_p(cubin)), "cuModuleLoadData")
    _check(cu.cuModuleGetFunction(C.byref(fn), mod, b"golden_march_dev"), "cuModuleGetFunction")
    os.makedirs(out_dir, exist_ok=True)
    for name, sc in SCENES.items():
        b = open(os.path.join(REF_DIR, f"golden_dev_{name}.bin"), "rb").read()
        srm, ssi = struct.unpack_from("<ii", b, 0)
        o = 8
        rm = np.frombuffer(b, np.uint8, srm, o)
        si = np.frombuffer(b, np.uint8, ssi, o + srm)
        o += srm + ssi
        n_pix, = struct.unpack_from("<i", b, o)
        pix = np.frombuffer(b, np.int32, 2 * n_pix, o + 4).reshape(-1, 2)
        o += 4 + 8 * n_pix
        max_steps, nlvl, nb = struct.unpack_from("<iii", b, o)
        o += 12
        assert nb == nlvl * 128 ** 3 // 8 and o + nb == len(b)
        bits = np.zeros((nlvl + 7) * 128 ** 3 // 8, np.uint8)  # zero pad: see the bounds note in the kernel
        bits[:nb] = np.frombuffer(b, np.uint8, nb, o)
        assert pix[:, 0].min() >= 0 and pix[:, 0].max() < sc["W"] and pix[:, 1].min() >= 0 and pix[:, 1].max() < sc["H"]
        d_rm = torch.from_numpy(rm.copy()).cuda()
        d_si = torch.from_numpy(si.copy()).cuda()
        d_bits = torch.from_numpy(bits).cuda()
        d_pix = torch.from_numpy(pix.copy()).cuda()
        d_out = torch.zeros(4 * n_pix, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        args = [C.c_void_p(d_rm.data_ptr()), C.c_void_p(d_si.data_ptr()), C.c_void_p(d_bits.data_ptr()),
                C.c_void_p(d_pix.data_ptr()), C.c_int(n_pix), C.c_int(max_steps), C.c_void_p(d_out.data_ptr())]
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        block = 128
        grid = (n_pix + block - 1) // block
        _check(cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, None, params, None), "cuLaunchKernel")
        _check(cu.cuCtxSynchronize(), "cuCtxSynchronize")
        out = d_out.cpu().numpy().reshape(-1, 4)
        s = STRIDE[name]
        gw, gh = (sc["W"] + s - 1) // s, (sc["H"] + s - 1) // s
        nd = gw * gh
        dense, gold = out[:nd], out[nd:]
        np.savez_compressed(os.path.join(out_dir, f"march_{name}_dev.npz"), stride=np.int32(s),
                            hits=dense[:, 0].astype(np.uint8).reshape(gh, gw),
                            steps=dense[:, 1].astype(np.int16).reshape(gh, gw),
                            occupied=dense[:, 2].astype(np.int16).reshape(gh, gw),
                            g_hits=gold[:, 0].astype(np.int32), g_steps=gold[:, 1].astype(np.int32),
                            g_occupied=gold[:, 2].astype(np.int32), g_t0_hash=gold[:, 3].astype(np.uint32))
        print(name, "rays", n_pix, "steps", int(dense[:, 1].sum()), "occupied", int(dense[:, 2].sum()),
              "max steps", int(out[:, 1].max()))
    cu.cuModuleUnload(mod)


if __name__ == "__main__":
    if len(sys.argv) >= 2 and sys.argv[1] == "prep":
        prep()
    elif len(sys.argv) == 3 and sys.argv[1] == "run":
        run(sys.argv[2])
    else:
        raise SystemExit(__doc__)
