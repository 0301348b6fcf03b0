"""The CPU oracle against an independent numpy restatement of the network,
and its renderers' invariants (no GPU)."""
import numpy as np
import pytest

from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import psnr, small_camera, tiny_model


@pytest.fixture(scope="module")
def om():
    return orc.OracleModel(tiny_model())


def test_hash_encoding_matches_numpy(om):
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 1, size=(2000, 3)).astype(np.float32)
    sm = fmodel.SyntheticModel(fmodel.spec_tiny())
    ref = fmodel.hash_encode(pos, sm.table.astype(np.float64), om.levels)
    got = om.hash_encode(pos)[:, :32]
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9)


def test_density_network_matches_numpy_fp16_path():
    o = orc.OracleModel(tiny_model(), mimic_fp16=True)
    sm = fmodel.SyntheticModel(fmodel.spec_tiny())
    rng = np.random.default_rng(4)
    pos = rng.uniform(0, 1, size=(500, 3)).astype(np.float32)
    d01 = rng.uniform(0, 1, size=(500, 3)).astype(np.float32)
    ref = sm.base_outputs(pos)[:, 0]
    got = o.inference(pos, d01)[:, 3]
    np.testing.assert_allclose(got, ref, atol=2e-3)


def test_plain_render_invariants(om):
    cam = small_camera(1001, 24, 20)
    res, ns, nst = om.render_plain(cam)
    T = res[..., 3]
    assert np.all(T > 0) and np.all(T <= 1)
    assert np.all(res[..., :3] >= 0) and np.all(res[..., :3] <= 1 + 1e-6)
    assert ns.max() > 0 and np.all(nst >= ns)


def test_cache_build_and_cached_render_self_consistent(om):
    cam = small_camera(1001, 32, 24)
    c = om.cache_build(cam)
    d = c.dims
    assert d.fW == 32 and d.fH == 24 and d.bX == 4 and d.bY == 3
    used = c.packed_index[c.packed_index >= 0]
    assert used.size == c.n_bricks_set > 0
    # slots are consecutive from 0 in (iteration, tile) order
    slots = np.sort(((used >> 20) & 1023) * (d.dY * d.dZ) + ((used >> 10) & 1023) * d.dZ + (used & 1023))
    np.testing.assert_array_equal(slots, np.arange(slots.size))
    plain, _, _ = om.render_plain(cam)
    cached, counts = om.render_cached(cam, c)
    hit = counts[..., 1].sum() / max(1, counts[..., :2].sum())
    assert hit > 0.5, hit
    assert psnr(cached[..., :3] + cached[..., 3:], plain[..., :3] + plain[..., 3:]) > 30


def test_view_dependent_network_matches_numpy_fp16_path():
    """The split network (NerfNetwork::init_viewdep, include/nerf_network.h:
    120-158) restated in numpy: density MLP, first head on [density outputs |
    SH of the initial direction], color head on [latents | SH | SH difference
    (zero for a row's own direction) | 1-padding], fp16 rounding per layer.
    Measured: 99.9 % of the logits identical, the rest one fp16 ulp apart
    (float64 summation order)."""
    spec = fmodel.spec_tiny(seed=31)
    spec.view_dependent, spec.name = True, f"{spec.name}_h2"
    o = orc.OracleModel(fmodel.ensure_model(spec), mimic_fp16=True)
    sm = fmodel.SyntheticModel(spec)
    rng = np.random.default_rng(6)
    pos = rng.uniform(0, 1, size=(400, 3)).astype(np.float32)
    d01 = rng.uniform(0, 1, size=(400, 3)).astype(np.float32)
    h16 = lambda x: x.astype(np.float16).astype(np.float64)  # noqa: E731
    W = lambda w: w.astype(np.float64)  # noqa: E731
    sh = h16(fmodel.sh4((d01 * np.float32(2) - np.float32(1)).astype(np.float64)))
    bo = sm.base_outputs(pos)                                       # [N, 16]
    f1 = h16(np.maximum(np.concatenate([bo, sh], axis=1) @ W(sm.first[0]).T, 0.0))
    fo = h16(f1 @ W(sm.first[1]).T)                                 # latents in rows 0..7
    n = pos.shape[0]
    x = np.concatenate([fo[:, :8], sh, np.zeros((n, 16)), np.ones((n, 8))], axis=1)
    for w in sm.head[:-1]:
        x = h16(np.maximum(x @ W(w).T, 0.0))
    ref = h16(x @ W(sm.head[-1]).T)[:, :3]
    got = o.inference(pos, d01)
    np.testing.assert_allclose(got[:, :3], ref, atol=1e-3)
    np.testing.assert_allclose(got[:, 3], bo[:, 0], atol=1e-12)


def test_four_feature_hash_encoding_matches_numpy():
    """The 8-level x 4-feature grid (instant-ngp's default): the oracle's
    encoding against the numpy restatement, features level-major."""
    import dataclasses
    spec = dataclasses.replace(fmodel.spec_tiny(seed=41), name="tiny41_f4", n_levels=8, F=4, per_level_scale=2.0)
    o = orc.OracleModel(fmodel.ensure_model(spec))
    sm = fmodel.SyntheticModel(spec)
    rng = np.random.default_rng(5)
    pos = rng.uniform(0, 1, size=(2000, 3)).astype(np.float32)
    ref = fmodel.hash_encode(pos, sm.table.astype(np.float64), o.levels, F=4)
    got = o.hash_encode(pos)[:, :32]
    assert ref.shape == (2000, 32)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9)
