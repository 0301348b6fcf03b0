"""The instant-ngp snapshot (.ingp) loader against the oracle's restatement of
load_ingp_snapshot (src/loader.cu:146-230).

CPU: the library's host-only reader (fvc_ingp_export: inflate, msgpack, the
derived scene / step / network configuration, the parameter split and the
occupancy threshold) writes the same nerfacc export as the oracle, byte for
byte, for every wrapper the reference's stream reader accepts (gzip, zlib with
stored, fixed-code and dynamic-code deflate blocks, none); the mean-density
threshold applies when the mean is below 0.01; malformed snapshots fail with
the reference's messages.  GPU: a snapshot loaded directly renders
bit-identically to its export, matches the oracle's render of the oracle's own
export within the parity tolerance, and reports DataSource INGP properties.
"""
import gzip
import json
import os

import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import _lib as L
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import ingp as oingp
from tests.ingp_fixture import density_grid, ingp_model, make_snapshot, pack, write_snapshot

BLOBS = ["pos_enc.dat", "mlp_base.dat", "mlp_head.dat", "occupancy_grid.dat"]


def _same_export(a, b):
    ca, cb = json.load(open(os.path.join(a, "config.json"))), json.load(open(os.path.join(b, "config.json")))

    def norm(v):
        if isinstance(v, dict):
            return {k: norm(x) for k, x in v.items()}
        if isinstance(v, list):
            return [norm(x) for x in v]
        if isinstance(v, float) or (isinstance(v, int) and not isinstance(v, bool)):
            return float(np.float32(v))
        return v

    assert norm(ca) == norm(cb)
    for n in BLOBS:
        assert open(os.path.join(a, n), "rb").read() == open(os.path.join(b, n), "rb").read(), n


@pytest.mark.parametrize("wrapper", ["gzip", "zlib", "stored", "fixed", "raw"])
def test_export_matches_oracle(tmp_path, wrapper):
    snap = make_snapshot(tmp_path, wrapper=wrapper)
    fvc.ingp_export(snap, tmp_path / "lib")
    cfg = oingp.snapshot_to_export(snap, str(tmp_path / "orc"))
    _same_export(tmp_path / "lib", tmp_path / "orc")
    sc = cfg["scene"]
    assert sc["grid_nlvl"] == 2 and sc["normalized"] and sc["cone_angle"] == float(np.float32(1 / 256))
    occ = np.fromfile(tmp_path / "lib" / "occupancy_grid.dat", np.uint8)
    _, _, _, _, occ0 = ingp_model(31, 2)
    # densities were drawn above 0.01 exactly where the source grid is occupied
    np.testing.assert_array_equal(occ, occ0)


def test_single_cascade_and_one_hidden_layer_head(tmp_path):
    spec, wb, wh, tab, occ = ingp_model(41, 1)
    wh1 = np.concatenate([wh[:64 * 32], wh[64 * 32 + 64 * 64:]])  # drop the second hidden layer
    dens = density_grid(occ, 1, 42)
    snap = write_snapshot(tmp_path / "one.ingp", 1, np.concatenate([wb, wh1, tab]), dens, head_hidden=1)
    fvc.ingp_export(snap, tmp_path / "lib")
    cfg = oingp.snapshot_to_export(snap, str(tmp_path / "orc"))
    _same_export(tmp_path / "lib", tmp_path / "orc")
    assert cfg["scene"]["cone_angle"] == 0.0 and cfg["mlp_head"]["network"]["n_hidden_layers"] == 1
    assert os.path.getsize(tmp_path / "lib" / "mlp_head.dat") == (64 * 32 + 16 * 64) * 2


def test_threshold_is_the_mean_when_below_001(tmp_path):
    snap = make_snapshot(tmp_path, low=True)
    fvc.ingp_export(snap, tmp_path / "lib")
    oingp.snapshot_to_export(snap, str(tmp_path / "orc"))
    _same_export(tmp_path / "lib", tmp_path / "orc")
    occ = np.fromfile(tmp_path / "lib" / "occupancy_grid.dat", np.uint8).reshape(2, -1)
    _, _, _, _, occ0 = ingp_model(31, 2)
    # a threshold of 0.01 would keep only cells drawn in (0.01, 0.05); the mean (~3e-3) keeps more
    dens = density_grid(occ0, 2, 32, low=True).astype(np.float32).reshape(2, -1)
    mean = np.maximum(dens[0], 0).astype(np.float64).mean()
    assert mean < 0.01
    assert occ[0].sum() == (dens[0] > np.float32(mean)).sum() > (dens[0] > 0.01).sum()


def test_per_level_scale_follows_the_aabb_scale(tmp_path):
    snap = make_snapshot(tmp_path, name="s4.ingp", seed=51, aabb_scale=4)
    fvc.ingp_export(snap, tmp_path / "lib")
    cfg = json.load(open(tmp_path / "lib" / "config.json"))
    b = cfg["mlp_base"]["encoding"]["per_level_scale"]
    assert abs(b - (2048.0 * 4 / 16) ** (1 / 15)) < 1e-6
    assert cfg["scene"]["grid_nlvl"] == 3 and cfg["scene"]["aabb"] == [-1.5, -1.5, -1.5, 2.5, 2.5, 2.5]
    oingp.snapshot_to_export(snap, str(tmp_path / "orc"))
    _same_export(tmp_path / "lib", tmp_path / "orc")


def _err(fn):
    with pytest.raises(L.FvcError) as e:
        fn()
    return str(e.value)


def test_malformed_snapshots_fail_with_the_reference_messages(tmp_path):
    spec, wb, wh, tab, occ = ingp_model(31, 2)
    params = np.concatenate([wb, wh, tab])
    dens = density_grid(occ, 2, 32)
    assert "Could not load snapshot file!" in _err(lambda: fvc.ingp_export(tmp_path / "missing.ingp", tmp_path / "o"))
    p = write_snapshot(tmp_path / "sdf.ingp", 2, params, dens, mode="sdf")
    assert "does not contain a nerf snapshot" in _err(lambda: fvc.ingp_export(p, tmp_path / "o"))
    p = tmp_path / "nosnap.ingp"
    p.write_bytes(gzip.compress(pack({"encoding": {}})))
    assert "does not contain a snapshot" in _err(lambda: fvc.ingp_export(p, tmp_path / "o"))
    good = open(write_snapshot(tmp_path / "t.ingp", 2, params, dens), "rb").read()
    (tmp_path / "trunc.ingp").write_bytes(good[: len(good) // 2])
    assert "deflate" in _err(lambda: fvc.ingp_export(tmp_path / "trunc.ingp", tmp_path / "o"))
    p = write_snapshot(tmp_path / "nogrid.ingp", 2, params, dens, drop=("density_grid_binary",))
    assert "density_grid_binary" in _err(lambda: fvc.ingp_export(p, tmp_path / "o"))
    p = write_snapshot(tmp_path / "short.ingp", 2, params[:1000], dens)
    assert "params_binary" in _err(lambda: fvc.ingp_export(p, tmp_path / "o"))
    p = write_snapshot(tmp_path / "grid.ingp", 2, params, dens[: len(dens) // 2])
    assert "density_grid_binary" in _err(lambda: fvc.ingp_export(p, tmp_path / "o"))


@pytest.mark.gpu
def test_snapshot_renders_like_its_export_and_the_oracle(tmp_path):
    from oracle import oracle as orc
    from tests.helpers import psnr, small_camera
    snap = make_snapshot(tmp_path, aabb_scale=2)
    exp = fvc.ingp_export(snap, tmp_path / "lib")
    oingp.snapshot_to_export(snap, str(tmp_path / "orc"))
    a, b = fvc.load_data(snap), fvc.load_data(exp)
    props = a.nerf_network.properties()
    assert props["first_latent_is_density"] and props["n_latents"] == 16
    assert a.data_source == "ingp" and b.data_source == "nerfacc"
    assert a.scene_info.normalized == 1 and b.scene_info.normalized == 1
    cam = small_camera(1201, 64, 48, radius=2.5)
    cam_c = dict(cam)
    cam_c["cam2world"] = np.asarray(cam["cam2world"], np.float32).copy()
    cam_c["cam2world"][:, 3] += 0.5  # orbit the unit cube's centre
    cam_c["world2cam"] = fcam.inverse(cam_c["cam2world"])
    outs = []
    for ld in (a, b):
        r = fvc.PerformanceRenderer(ld.scene_info, ld.occupancy_grid_morton_bitfield, ld.nerf_network)
        r.resizeRenderbuffers(cam_c["resolution"])
        buf = fvc.RenderBuffer(cam_c["resolution"])
        r.render(fvc.raymarch_info(cam_c, ld.stepsize_info), buf)
        outs.append((buf.results.copy(), buf.ray_counts.copy()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    om = orc.OracleModel(str(tmp_path / "orc"))
    ref, ns, _ = om.render_plain(cam_c)
    np.testing.assert_array_equal(outs[0][1][..., 0], ns)
    assert ns.sum() > 1000
    err = np.abs(outs[0][0] - ref).max()
    p = psnr(outs[0][0][..., :3] + outs[0][0][..., 3:], ref[..., :3] + ref[..., 3:])
    print(f"\n.ingp plain 64x48: max-abs {err:.2e}, PSNR vs fp64 oracle {p:.1f} dB, samples {ns.sum()}")
    assert err <= 2e-3
    # the snapshot's head reads 16 latents, a cache voxel holds 8: the cache renderer refuses it
    c0, c1 = fvc.Cache(), fvc.Cache()
    rc = fvc.CachePerformanceRenderer(a.scene_info, a.occupancy_grid_morton_bitfield, a.nerf_network, c0, c1)
    rc.resizeCache(cam_c["resolution"], a.stepsize_info)
    rc.resizeRenderbuffers(cam_c["resolution"])
    rc.setCacheSettings(fvc.eval_cache_settings(a))
    with pytest.raises(fvc._lib.FvcError) as e:
        rc.initCacheBlockwise(fvc.raymarch_info(cam_c, a.stepsize_info))
    assert e.value.code == 2 and "8 latents" in str(e.value)


def test_eight_level_four_feature_grid_exports_like_the_oracle(tmp_path):
    """instant-ngp's default grid (8 levels x 4 features): the snapshot's
    parameter split and export match the oracle's restatement."""
    import dataclasses
    spec, wb, wh, _, occ = ingp_model(51, 2)
    spec = dataclasses.replace(spec, name="ingp_like51_f4", n_levels=8, F=4,
                               per_level_scale=float((2048.0 * 2 / 16.0) ** (1.0 / 7.0)))
    tab = fmodel.SyntheticModel(spec).table.ravel().view(np.uint16)
    dens = density_grid(occ, 2, 52)
    snap = write_snapshot(tmp_path / "f4.ingp", 2, np.concatenate([wb, wh, tab]), dens, n_levels=8, n_features=4)
    fvc.ingp_export(snap, tmp_path / "lib")
    cfg = oingp.snapshot_to_export(snap, str(tmp_path / "orc"))
    _same_export(tmp_path / "lib", tmp_path / "orc")
    enc = cfg["mlp_base"]["encoding"]
    assert enc["n_levels"] == 8 and enc["n_features_per_level"] == 4
    assert os.path.getsize(tmp_path / "lib" / "pos_enc.dat") == tab.size * 2
