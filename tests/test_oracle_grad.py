"""The oracle's float64 adjoint of the differentiable render against float64
central finite differences (h = 1e-4) of its own loss.

This pins the compositing adjoint (dL/dsigma in sample order from the prefix
of T alpha g.c) and the network adjoint (dense layers, ReLU, the hash-grid
scatter) that the GPU gradients are later compared with.  The loss is
piecewise smooth: a perturbation can cross a ReLU kink or move the early
termination, so the check asks that nearly all sampled parameters agree
tightly and the sampled gradient vectors agree as a whole.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import small_camera, tiny_model

H_FD = 1e-4


@pytest.fixture(scope="module")
def case():
    om = orc.OracleModel(tiny_model(7, 1), mimic_fp16=False)
    W = H = 24
    cam = small_camera(1001, W, H)
    rng = np.random.default_rng(5)
    pix = rng.choice(W * H, 64, replace=False).astype(np.int32)
    tgt = rng.uniform(0, 1, (64, 3)).astype(np.float32)
    loss, gt, gb, gh, pred = om.loss_grad(cam, pix, tgt)
    return om, cam, pix, tgt, loss, (gt, gb, gh), pred, rng


def test_loss_matches_the_plain_render(case):
    om, cam, pix, tgt, loss, _, pred, _ = case
    res, _, _ = om.render_plain(cam)
    img = res.reshape(-1, 4)[pix]
    np.testing.assert_allclose(pred, img, atol=1e-6)
    expect = np.mean(np.sum((img[:, :3] + img[:, 3:4] - tgt) ** 2, axis=1))
    assert abs(loss - expect) < 1e-6


@pytest.mark.parametrize("group", [0, 1, 2], ids=["hash_table", "density_mlp", "color_head"])
def test_adjoint_matches_central_differences(case, group):
    om, cam, pix, tgt, _, grads, _, rng = case
    g = grads[group]
    nz = np.flatnonzero(g)
    assert nz.size > 100
    pick = rng.choice(nz, 86, replace=False)  # 3 groups x 86 = 258 sampled parameters
    fd = []
    for k in pick:
        lp = om.loss_grad(cam, pix, tgt, grads=False, perturb=([group], [k], [H_FD]))[0]
        lm = om.loss_grad(cam, pix, tgt, grads=False, perturb=([group], [k], [-H_FD]))[0]
        fd.append((lp - lm) / (2 * H_FD))
    fd = np.array(fd)
    an = g[pick]
    rel = np.abs(an - fd) / np.maximum(np.abs(fd), 1e-9)
    # kink crossings at h = 1e-4 (ReLU, early termination) move a minority of
    # entries by up to a few percent; the bulk agrees to < 1e-4
    assert np.median(rel) < 1e-4, rel
    assert np.mean(rel < 1e-3) >= 0.75, rel
    assert np.mean(rel < 5e-2) >= 0.95, rel
    cos = float(an @ fd / (np.linalg.norm(an) * np.linalg.norm(fd)))
    assert cos > 0.9999


def test_cached_adjoint_latents_match_central_differences():
    """The cached render's adjoint with respect to the cache brick latents
    (cache rows blend the 8 corner latents with w_c / sum(w isset)) against
    central differences of the oracle's own cached loss."""
    om = orc.OracleModel(tiny_model(7, 1), mimic_fp16=False)
    W = H = 24
    cam = small_camera(1001, W, H)
    cache = om.cache_build(cam)
    rng = np.random.default_rng(8)
    pix = rng.choice(W * H, 64, replace=False).astype(np.int32)
    tgt = rng.uniform(0, 1, (64, 3)).astype(np.float32)
    loss, gt, gb, gh, gl, pred = om.loss_grad_cached(cam, cache, pix, tgt)
    res, _ = om.render_cached(cam, cache)
    np.testing.assert_allclose(pred, res.reshape(-1, 4)[pix], atol=1e-6)
    nz = np.flatnonzero(gl)
    assert nz.size > 100 and np.count_nonzero(gh) > 100
    pick = rng.choice(nz, 86, replace=False)
    fd = np.array([(om.loss_grad_cached(cam, cache, pix, tgt, grads=False, perturb=([k], [H_FD]))[0] -
                    om.loss_grad_cached(cam, cache, pix, tgt, grads=False, perturb=([k], [-H_FD]))[0]) / (2 * H_FD)
                   for k in pick])
    an = gl[pick]
    rel = np.abs(an - fd) / np.maximum(np.abs(fd), 1e-9)
    assert np.median(rel) < 1e-4, rel
    assert np.mean(rel < 1e-3) >= 0.75, rel
    cos = float(an @ fd / (np.linalg.norm(an) * np.linalg.norm(fd)))
    assert cos > 0.9999
