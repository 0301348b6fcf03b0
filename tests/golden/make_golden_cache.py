"""Regenerates tests/golden/cache_build.npz from the reference's own cache-build
kernels run on the host: the blockwise build (initPayloads_cache_init_kernel
through writeImageBuffer_cache_init_kernel2, src/cache_renderer.cu:18-569,
under the host loop of CacheRenderer::initCacheBlockwise, :931-1041) by
oracle/_ref/libref_cache_build.so, and the per-ray fill (the payload,
compaction and sampling kernels of src/renderer.cu and
accumulate_cache_init_first_kernel .. writeImageBuffer_cache_init_kernel,
src/cache_renderer.cu:571-830, under CacheRenderer::initCache, :848-928) by
oracle/_ref/libref_cache_fill.so (oracle/Makefile, target ``ref``).

Run from the repository root where the reference tree is available:
    make -C oracle ref REF=<reference checkout>
    python tests/golden/make_golden_cache.py

The network between the kernels (NerfNetwork::inferenceLatents) is the
float64 oracle's density network at the kernels' own sample positions,
rounded to float and then to fp16, as a network with float accumulators
stores its outputs.  Cases: the
small synthetic models of the tests (three cascades with L-inf contraction
and cone 1/256; one cascade with cone 0) at 24x16 and 16x16, built at seeded
camera poses inside the scene box, with the Density and Alpha variants.  The data
arrays hold every brick (no overflow), so the set of bricks with a slot is
deterministic; the slots themselves come from the reference's atomicAdd and
are not recorded, only each brick's voxels.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_cache_build.so")
FILL_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_cache_fill.so")

# (name, model seed, cascades, camera seed, camera radius, W, H, interpol_variant); the cameras lie inside the
# scene box: the reference sizes the frustum depth for that (resizeCache) and writes past its brick arrays otherwise
CASES = [
    ("c3_density", 9, 3, 2102, 4.0, 24, 16, 0),
    ("c3_alpha", 9, 3, 2103, 3.0, 24, 16, 1),
    ("c1_density", 7, 1, 2101, 1.2, 16, 16, 0),
]


def case_inputs(seed, nlvl, cam_seed, radius, W, H):
    from frustumvolumecaching_gb300 import camera as fcam
    from frustumvolumecaching_gb300 import model as fmodel
    from oracle import oracle as orc

    d = fmodel.ensure_model(fmodel.spec_tiny(seed=seed, nlvl=nlvl))
    om = orc.OracleModel(d)
    cam = fcam.seeded_camera(cam_seed, radius=radius, width=W, height=H)
    return om, cam


def scene_params(om, cam):
    """The plain parameters rcb_init builds the reference structs from."""
    sc = om.cfg["scene"]
    warp = "contraction" in sc and "aabb" in sc["contraction"]  # L-inf warp about the contraction box, else the AABB
    cfa = sc["contraction"]["aabb"] if warp else sc["aabb"]
    contraction = 1 if warp else 0
    c2w = np.asarray(cam["cam2world"], np.float32).reshape(3, 4)
    f = np.zeros(33, np.float32)
    f[0:6] = sc["aabb"]
    f[6:12] = cfa
    f[12:17] = [sc["cone_angle"], sc["stepsize"], sc["near"], sc["far"], sc.get("alpha_thre", 0.0)]
    f[17:19] = cam["focal"]
    f[19:21] = cam["principal"]
    f[21:33] = c2w.ravel()
    return np.asarray([om.scene.grid_nlvl, contraction], np.int32), f


def run_case(lib, om, cam, W, H, variant):
    sci, f = scene_params(om, cam)
    dims = om.cache_dims(W, H)
    data_bricks = np.asarray([dims.dX, dims.dY, dims.dZ], np.int32)
    lo = int(om.net.latent_offset)
    n_tiles = lib.rcb_init(sci.ctypes.data, f.ctypes.data, W, H, om.bits.ctypes.data, data_bricks.ctypes.data, lo, variant)
    assert n_tiles > 0
    fr = np.zeros(6, np.int32)
    lib.rcb_dims(fr.ctypes.data)
    iters = 0
    while True:
        pp, tp = C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
        n = lib.rcb_search(C.byref(pp), C.byref(tp))
        if n <= 0:
            break
        pos = np.ctypeslib.as_array(pp, shape=(n * 3,)).reshape(n, 3).copy()
        dir01 = np.full((n, 3), 0.5, np.float32)  # unused by a model without a first head
        bo = om.base_outputs(pos, dir01)
        batch = (n + 255) // 256 * 256  # tcnn::next_multiple(n, batch_size_granularity)
        out = np.zeros((bo.shape[1], batch), np.float16)
        out[:, :n] = bo.T.astype(np.float32).astype(np.float16)  # a float accumulator rounded to the stored half
        assert lib.rcb_accumulate(out.view(np.uint16).ctypes.data, batch) == 0
        iters += 1
    bX, bY, bZ = int(fr[3]), int(fr[4]), int(fr[5])
    packed = np.zeros(bX * bY * bZ, np.int32)
    known = np.zeros(int(fr[0]) * int(fr[1]), np.float32)
    oob = C.c_longlong(0)
    demanded = lib.rcb_finish(packed.ctypes.data, known.ctypes.data, C.byref(oob))
    n_set = int((packed >= 0).sum())
    isset = np.zeros((n_set, 512), np.float32)
    dens = np.zeros((n_set, 512), np.float32)
    lat = np.zeros((n_set, 512, 8), np.uint16)
    assert lib.rcb_bricks(isset.ctypes.data, dens.ctypes.data, lat.ctypes.data) == n_set
    vox = isset > 0
    return {
        "frustum": fr[:3].copy(), "bricks": fr[3:].copy(), "brick_set": (packed >= 0).astype(np.uint8),
        "known": known.reshape(int(fr[1]), int(fr[0])), "demanded": np.int32(demanded), "iterations": np.int32(iters),
        "out_of_range_writes": np.int64(oob.value), "isset": np.packbits(vox, axis=1),
        "density": dens[vox], "latents": lat[vox], "variant": np.int32(variant),
    }


def run_fill_case(lib, om, cam, W, H, variant):
    """The per-ray fill (CacheRenderer::initCache, src/cache_renderer.cu:848-928) through the reference's
    kernels in oracle/_ref/libref_cache_fill.so; the same outputs as run_case."""
    sci, f = scene_params(om, cam)
    dims = om.cache_dims(W, H)
    data_bricks = np.asarray([dims.dX, dims.dY, dims.dZ], np.int32)
    assert lib.rcf_init(sci.ctypes.data, f.ctypes.data, W, H, om.bits.ctypes.data, data_bricks.ctypes.data,
                        int(om.net.latent_offset), variant) == W * H
    fr = np.zeros(6, np.int32)
    lib.rcf_dims(fr.ctypes.data)
    iters = 0
    while True:
        pp = C.POINTER(C.c_float)()
        batch = C.c_int(0)
        rows = lib.rcf_search(C.byref(pp), C.byref(batch))
        if rows <= 0:
            break
        pos = np.ctypeslib.as_array(pp, shape=(rows * 3,)).reshape(rows, 3).copy()
        bo = om.base_outputs(pos, np.full((rows, 3), 0.5, np.float32))
        out = np.zeros((bo.shape[1], batch.value), np.float16)
        out[:, :rows] = bo.T.astype(np.float32).astype(np.float16)
        assert lib.rcf_accumulate(out.view(np.uint16).ctypes.data) == 0
        iters += 1
    bX, bY, bZ = int(fr[3]), int(fr[4]), int(fr[5])
    packed = np.zeros(bX * bY * bZ, np.int32)
    known = np.zeros(int(fr[0]) * int(fr[1]), np.float32)
    oob = C.c_longlong(0)
    demanded = lib.rcf_finish(packed.ctypes.data, known.ctypes.data, C.byref(oob))
    n_set = int((packed >= 0).sum())
    isset = np.zeros((n_set, 512), np.float32)
    dens = np.zeros((n_set, 512), np.float32)
    lat = np.zeros((n_set, 512, 8), np.uint16)
    assert lib.rcf_bricks(isset.ctypes.data, dens.ctypes.data, lat.ctypes.data) == n_set
    vox = isset > 0
    return {
        "frustum": fr[:3].copy(), "bricks": fr[3:].copy(), "brick_set": (packed >= 0).astype(np.uint8),
        "known": known.reshape(int(fr[1]), int(fr[0])), "demanded": np.int32(demanded), "iterations": np.int32(iters),
        "out_of_range_writes": np.int64(oob.value), "isset": np.packbits(vox, axis=1),
        "density": dens[vox], "latents": lat[vox], "variant": np.int32(variant),
    }


def main():
    lib = C.CDLL(LIB)
    V, I = C.c_void_p, C.c_int
    lib.rcb_init.argtypes = [V, V, I, I, V, V, I, I]
    lib.rcb_dims.argtypes = [V]
    lib.rcb_search.argtypes = [C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.POINTER(C.c_float))]
    lib.rcb_accumulate.argtypes = [V, I]
    lib.rcb_finish.argtypes = [V, V, C.POINTER(C.c_longlong)]
    lib.rcb_bricks.argtypes = [V, V, V]
    for fn in (lib.rcb_init, lib.rcb_search, lib.rcb_accumulate, lib.rcb_finish, lib.rcb_bricks):
        fn.restype = I
    arrays = {}
    for name, seed, nlvl, cam_seed, radius, W, H, variant in CASES:
        om, cam = case_inputs(seed, nlvl, cam_seed, radius, W, H)
        r = run_case(lib, om, cam, W, H, variant)
        for k, v in r.items():
            arrays[f"{name}/{k}"] = v
        print(f"{name}: {int(r['brick_set'].sum())} bricks, {int(r['demanded'])} demanded, {int(r['iterations'])} iterations, "
              f"{r['density'].size} voxels set, {int(r['out_of_range_writes'])} out-of-range writes")
    fill = C.CDLL(FILL_LIB)
    fill.rcf_init.argtypes = [V, V, I, I, V, V, I, I]
    fill.rcf_dims.argtypes = [V]
    fill.rcf_search.argtypes = [C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.c_int)]
    fill.rcf_accumulate.argtypes = [V]
    fill.rcf_finish.argtypes = [V, V, C.POINTER(C.c_longlong)]
    fill.rcf_bricks.argtypes = [V, V, V]
    for fn in (fill.rcf_init, fill.rcf_search, fill.rcf_accumulate, fill.rcf_finish, fill.rcf_bricks):
        fn.restype = I
    for name, seed, nlvl, cam_seed, radius, W, H, variant in CASES:
        om, cam = case_inputs(seed, nlvl, cam_seed, radius, W, H)
        r = run_fill_case(fill, om, cam, W, H, variant)
        for k, v in r.items():
            arrays[f"fill_{name}/{k}"] = v
        print(f"per-ray fill {name}: {int(r['brick_set'].sum())} bricks, {int(r['demanded'])} demanded, "
              f"{int(r['iterations'])} iterations, {r['density'].size} voxels set, {int(r['out_of_range_writes'])} out-of-range writes")
    np.savez_compressed(os.path.join(HERE, "cache_build.npz"), **arrays)


if __name__ == "__main__":
    main()
