"""The oracle's cache builds against golden vectors from the reference's own
build kernels (tests/golden/cache_build.npz, made by
tests/golden/make_golden_cache.py: the blockwise build from
initPayloads_cache_init_kernel .. writeImageBuffer_cache_init_kernel2,
src/cache_renderer.cu:18-569; the per-ray fill from the payload, compaction
and sampling kernels of src/renderer.cu and src/cache_renderer.cu:571-830;
with the oracle's density network rounded to fp16 between them).

Compared per case (no overflow, so the reference's set of bricks is
deterministic; its slots come from atomicAdd and are not compared):
  - which frustum bricks hold a slot, the bricks demanded: exact;
  - the known ranges (t at each tile's final depth brick): bit-exact with
    the step grid's transcendentals from the host libm, as the reference's
    kernels ran here; within 2 ulp with the oracle's own (the product's,
    fvc_detmath.h);
  - per brick, which voxels are set: exact; their 8 latents: the same fp16
    bits (the oracle rounds the same float64 outputs once);
  - their density slot: within the fp16 rounding of the log-density the
    reference's kernel reads (the oracle keeps it in float64)."""
import os

import numpy as np
import pytest

from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "cache_build.npz")

# the cases of tests/golden/make_golden_cache.py
CASES = [
    ("c3_density", 9, 3, 2102, 4.0, 24, 16, 0),
    ("c3_alpha", 9, 3, 2103, 3.0, 24, 16, 1),
    ("c1_density", 7, 1, 2101, 1.2, 16, 16, 0),
]


BUILDS = ["blockwise", "per_ray"]


def _build(om, cam, variant, builder):
    return om.cache_build(cam, variant=variant) if builder == "blockwise" else om.cache_build_per_ray(cam, variant=variant)


@pytest.mark.parametrize("builder", BUILDS)
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_cache_build_matches_reference_kernels(case, builder):
    """the blockwise build against initPayloads_cache_init_kernel ..
    writeImageBuffer_cache_init_kernel2, the per-ray fill against the
    payload, compaction and sampling kernels and accumulate_cache_init_*,
    reserveNewBricks_kernel and writeImageBuffer_cache_init_kernel"""
    from oracle import oracle as orc

    case_name, seed, nlvl, cam_seed, radius, W, H, variant = case
    name = case_name if builder == "blockwise" else "fill_" + case_name
    g = np.load(GOLDEN)
    om = orc.OracleModel(fmodel.ensure_model(fmodel.spec_tiny(seed=seed, nlvl=nlvl)), use_libm=True)
    cam = fcam.seeded_camera(cam_seed, radius=radius, width=W, height=H)
    cc = _build(om, cam, variant, builder)
    d = cc.dims
    assert [d.fW, d.fH, d.fD] == g[f"{name}/frustum"].tolist()
    assert [d.bX, d.bY, d.bZ] == g[f"{name}/bricks"].tolist()
    assert int(g[f"{name}/out_of_range_writes"]) == 0
    ref_set = g[f"{name}/brick_set"].astype(bool)
    np.testing.assert_array_equal(cc.packed_index >= 0, ref_set)
    assert cc.n_demanded == int(g[f"{name}/demanded"]) == int(ref_set.sum())
    np.testing.assert_array_equal(cc.known_ranges.view(np.uint32), g[f"{name}/known"].reshape(-1).view(np.uint32))
    # the oracle's voxels of each set brick, in brick-cell order (the golden's order)
    p = cc.packed_index[ref_set]
    sx, sy, sz = (p >> 20) & 1023, (p >> 10) & 1023, p & 1023
    slots = (sx * d.dY + sy) * d.dZ + sz
    vox = (slots[:, None] * 512 + np.arange(512)[None, :]).reshape(-1)
    isset = cc.vox_isset[vox].reshape(-1, 512) > 0
    ref_isset = np.unpackbits(g[f"{name}/isset"], axis=1, count=512).astype(bool)
    np.testing.assert_array_equal(isset, ref_isset)
    lat = cc.vox_latents.reshape(-1, 8)[vox[isset.reshape(-1)]]
    np.testing.assert_array_equal(lat, g[f"{name}/latents"])
    dens = cc.vox_density[vox[isset.reshape(-1)]]
    np.testing.assert_allclose(dens, g[f"{name}/density"], rtol=2e-3, atol=1e-6)
    # the same build on the oracle's own step-grid arithmetic: the same bricks and voxels, known ranges within 2 ulp
    own = _build(orc.OracleModel(fmodel.ensure_model(fmodel.spec_tiny(seed=seed, nlvl=nlvl))), cam, variant, builder)
    np.testing.assert_array_equal(own.packed_index >= 0, ref_set)
    ulp = np.abs(own.known_ranges.view(np.int32).astype(np.int64) - g[f"{name}/known"].reshape(-1).view(np.int32).astype(np.int64))
    assert int(ulp.max()) <= 2


@pytest.mark.gpu
@pytest.mark.parametrize("builder", BUILDS)
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_device_cache_build_matches_reference_kernels(case, builder):
    """The device's blockwise build against the same golden vectors: which
    bricks hold a slot, the bricks demanded and each brick's set voxels
    exactly; known ranges within 2 ulp (the device's step grid uses
    fvc_detmath.h, the golden run libm); latents and densities within fp16
    rounding (the device's network accumulates in float32, the golden's
    outputs are the float64 network rounded)."""
    import frustumvolumecaching_gb300 as fvc

    case_name, seed, nlvl, cam_seed, radius, W, H, variant = case
    name = case_name if builder == "blockwise" else "fill_" + case_name
    g = np.load(GOLDEN)
    loader = fvc.load_data(fmodel.ensure_model(fmodel.spec_tiny(seed=seed, nlvl=nlvl)))
    cam = fcam.seeded_camera(cam_seed, radius=radius, width=W, height=H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.setCacheSettings(fvc.default_cache_settings(variant))
    r.resizeRenderbuffers((W, H))
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    if builder == "blockwise":
        r.initCacheBlockwise(info)
    else:
        r.initCache(info)
    packed, known, vox = c1.read()
    ref_set = g[f"{name}/brick_set"].astype(bool)
    np.testing.assert_array_equal(packed.ravel() >= 0, ref_set)
    assert r._init_stats.n_bricks_demanded == int(g[f"{name}/demanded"])
    ulp = np.abs(known.ravel().view(np.int32).astype(np.int64) - g[f"{name}/known"].reshape(-1).view(np.int32).astype(np.int64))
    assert int(ulp.max()) <= 2
    p = packed.ravel()[ref_set]
    _, _, (dX, dY, dZ) = c1.dims()
    slots = (((p >> 20) & 1023) * dY + ((p >> 10) & 1023)) * dZ + (p & 1023)
    v = vox.reshape(-1, 512, 8)[slots]  # [bricks, 512, 8] u32 words: density, isset, 2 pad, 8 fp16 latents
    isset = v[..., 1].view(np.float32) > 0
    np.testing.assert_array_equal(isset, np.unpackbits(g[f"{name}/isset"], axis=1, count=512).astype(bool))
    lat = np.ascontiguousarray(v[..., 4:8][isset]).view(np.uint16).reshape(-1, 8).view(np.float16).astype(np.float32)
    ref_lat = g[f"{name}/latents"].view(np.float16).astype(np.float32)
    assert float(np.abs(lat - ref_lat).max()) < 2e-3
    dens = v[..., 0].view(np.float32)[isset]
    np.testing.assert_allclose(dens, g[f"{name}/density"], rtol=2e-3, atol=1e-6)
