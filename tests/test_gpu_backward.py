"""GPU adjoint of the plain render against the oracle's float64 adjoint.

The oracle's adjoint is pinned to central finite differences
(test_oracle_grad.py); here the device gradients of the same loss (hash
table, density MLP, color head) are compared with it on the same rays, with
the oracle rounding activations to fp16 like the device.  Tolerances: the
loss within 1e-4 relative; per parameter group a cosine similarity above
0.9999 and a relative L2 error below 2e-3 (measured on a GB300: table 8e-5,
density MLP 5e-6, color head 4e-6; against the oracle without fp16 rounding
2.7e-3 / 1.2e-4 / 1.0e-4).  Also checked: gradients accumulate across calls and
fvc_grad_zero clears them; the tcgen05 and mma.sync forward paths give the
same gradients.
"""
import numpy as np
import pytest

import frustumvolumecaching_gb300 as fvc
from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import small_camera, tiny_model

pytestmark = pytest.mark.gpu


def _case(seed=7, W=32, H=32, n=384):
    torch = pytest.importorskip("torch")
    d = tiny_model(seed, 1)
    loader = fvc.load_data(d)
    cam = small_camera(1001, W, H)
    rng = np.random.default_rng(11)
    pix = rng.choice(W * H, n, replace=False).astype(np.int32)
    tgt = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    return torch, d, loader, cam, pix, tgt


def _gpu(torch, loader, cam, pix, tgt, tcgen05=True, grads=None, calls=1, precision=0):
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    r.set_network_path(tcgen05)
    r.set_precision(precision)
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    g = grads or fvc.Gradients(loader.nerf_network)
    dp = torch.from_numpy(pix).cuda()
    dt = torch.from_numpy(tgt).cuda()
    pred = torch.zeros((pix.size, 4), dtype=torch.float32, device="cuda")
    loss = None
    for _ in range(calls):
        loss = r.render_backward(info, dp, dt, g, pred=pred)
    return loss, g, pred.cpu().numpy()


def _compare(a, b):
    cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
    rel = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return cos, rel


def test_backward_matches_oracle_adjoint():
    torch, d, loader, cam, pix, tgt = _case()
    loss, g, pred = _gpu(torch, loader, cam, pix, tgt)
    om = orc.OracleModel(d, mimic_fp16=True)
    oloss, ot, ob, oh, opred = om.loss_grad(cam, pix, tgt)
    assert abs(loss - oloss) <= 1e-4 * oloss
    assert np.abs(pred - opred).max() < 2e-3
    gt, gb, gh = g.read()
    for name, a, b in (("table", gt, ot), ("base", gb, ob), ("head", gh, oh)):
        cos, rel = _compare(a.astype(np.float64), b)
        assert cos > 0.9999 and rel < 2e-3, (name, cos, rel)


def test_gradients_accumulate_and_zero():
    torch, d, loader, cam, pix, tgt = _case(n=128)
    _, g1, _ = _gpu(torch, loader, cam, pix, tgt)
    one = [x.copy() for x in g1.read()]
    _gpu(torch, loader, cam, pix, tgt, grads=g1)
    two = g1.read()
    for a, b in zip(one, two):
        np.testing.assert_allclose(b, 2 * a, rtol=1e-4, atol=1e-9)
    g1.zero()
    assert all(not x.any() for x in g1.read())


def test_backward_same_on_both_forward_paths():
    torch, d, loader, cam, pix, tgt = _case(n=256)
    l1, g1, _ = _gpu(torch, loader, cam, pix, tgt, tcgen05=True)
    l2, g2, _ = _gpu(torch, loader, cam, pix, tgt, tcgen05=False)
    assert abs(l1 - l2) <= 1e-4 * l2
    for a, b in zip(g1.read(), g2.read()):
        cos, rel = _compare(a.astype(np.float64), b.astype(np.float64))
        assert cos > 0.999 and rel < 0.05


def test_bf16_backward_against_float64_adjoint():
    """BF16 MLPs (forward on tcgen05 kind::f16 with bf16 operands, backward on
    bf16 mma.sync) against the float64 adjoint without fp16 rounding."""
    torch, d, loader, cam, pix, tgt = _case()
    loss, g, _ = _gpu(torch, loader, cam, pix, tgt, precision=fvc.PerformanceRenderer.BF16)
    oloss, ot, ob, oh, _ = orc.OracleModel(d, mimic_fp16=False).loss_grad(cam, pix, tgt)
    assert abs(loss - oloss) <= 1e-3 * oloss
    for name, a, b in zip(("table", "base", "head"), g.read(), (ot, ob, oh)):
        cos, rel = _compare(a.astype(np.float64), b)
        print(f"bf16 {name}: cos {cos:.6f} rel {rel:.3e}")
        assert cos > 0.999 and rel < 3e-2, (name, cos, rel)  # measured: table 1.1e-2, base 8e-4, head 4e-3


def test_fp8_backward_is_refused():
    torch, d, loader, cam, pix, tgt = _case(n=32)
    with pytest.raises(fvc._lib.FvcError):
        _gpu(torch, loader, cam, pix, tgt, precision=fvc.PerformanceRenderer.FP8_E4M3)


def test_cached_backward_with_latent_gradients():
    """Adjoint of the cached render: hash table and MLP gradients from the
    resampled rows, head and cache-latent gradients from the cache rows,
    against the oracle's cached adjoint over the same (device-built) cache."""
    torch = pytest.importorskip("torch")
    d = tiny_model(7, 1)
    loader = fvc.load_data(d)
    W = H = 32
    cam0 = small_camera(1001, W, H)
    c0, c1 = fvc.Cache(), fvc.Cache()
    r = fvc.CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network, c0, c1)
    r.resizeCache((W, H), loader.stepsize_info)
    r.resizeRenderbuffers((W, H))
    r.setCacheSettings(fvc.default_cache_settings())
    r.initCacheBlockwise(fvc.raymarch_info(cam0, loader.stepsize_info))
    r.swapCache()
    # render from a view rotated by 1 degree: both resample and cache rows
    c2w = np.asarray(cam0["cam2world"], np.float64)
    a = np.radians(1.0)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    cam1 = fcam.camera_dict(np.concatenate([R @ c2w[:, :3], (R @ c2w[:, 3])[:, None]], axis=1), W, H)
    rng = np.random.default_rng(12)
    pix = rng.choice(W * H, 384, replace=False).astype(np.int32)
    tgt = rng.uniform(0, 1, (384, 3)).astype(np.float32)
    g = fvc.Gradients(loader.nerf_network)
    pred = torch.zeros((pix.size, 4), dtype=torch.float32, device="cuda")
    loss = r.render_backward(fvc.raymarch_info(cam1, loader.stepsize_info), torch.from_numpy(pix).cuda(),
                             torch.from_numpy(tgt).cuda(), g, pred=pred)
    om = orc.OracleModel(d, mimic_fp16=True)
    oc = orc.OracleCache(om.cache_dims(W, H), cam0)
    oc.load_device_cache(*c1.read())  # built into c1, the current cache after the swap
    oloss, ot, ob, oh, ol, opred = om.loss_grad_cached(cam1, oc, pix, tgt)
    assert abs(loss - oloss) <= 1e-4 * oloss
    assert np.abs(pred.cpu().numpy() - opred).max() < 2e-3
    gl = g.cache_latents().reshape(-1)
    assert np.count_nonzero(ol) > 100
    for name, a_, b_ in zip(("table", "base", "head", "latents"), (*g.read(), gl), (ot, ob, oh, ol[:gl.size])):
        cos, rel = _compare(a_.astype(np.float64), b_)
        print(f"cached {name}: cos {cos:.6f} rel {rel:.3e}")
        assert cos > 0.9999 and rel < 2e-3, (name, cos, rel)  # measured: 1.5e-4 / 1.6e-5 / 5.4e-6 / 3.6e-4


@pytest.mark.parametrize("tcgen05", [True, False], ids=["tcgen05", "mma_sync"])
def test_backward_one_hidden_layer_head(tcgen05):
    """A color head with one hidden layer (the tcgen05 adjoint's HH = 1 form:
    the output-layer gradient is masked by head hidden 1 directly)."""
    torch = pytest.importorskip("torch")
    spec = fmodel.spec_tiny(seed=21)
    spec.name, spec.head_hidden_layers = f"{spec.name}_h1", 1
    d = fmodel.ensure_model(spec)
    loader = fvc.load_data(d)
    cam = small_camera(1001, 32, 32)
    rng = np.random.default_rng(13)
    pix = rng.choice(32 * 32, 384, replace=False).astype(np.int32)
    tgt = rng.uniform(0, 1, (384, 3)).astype(np.float32)
    loss, g, _ = _gpu(torch, loader, cam, pix, tgt, tcgen05=tcgen05)
    oloss, ot, ob, oh, _ = orc.OracleModel(d, mimic_fp16=True).loss_grad(cam, pix, tgt)
    assert abs(loss - oloss) <= 1e-4 * oloss
    for name, a, b in zip(("table", "base", "head"), g.read(), (ot, ob, oh)):
        cos, rel = _compare(a.astype(np.float64), b)
        print(f"one-hidden-layer head {name}: cos {cos:.6f} rel {rel:.3e}")
        assert cos > 0.9999 and rel < 2e-3, (name, cos, rel)


H_FD = 1e-4      # central-difference step of the float64 oracle loss
SMOOTH = 1e-4    # an entry is smooth when its differences at h and h/2 agree to this (relative)
FD_REL = 1e-3    # the gradient bound


def _fd(om, cam, pix, tgt, group, k):
    def d(h):
        lp = om.loss_grad(cam, pix, tgt, grads=False, perturb=([group], [k], [h]))[0]
        lm = om.loss_grad(cam, pix, tgt, grads=False, perturb=([group], [k], [-h]))[0]
        return (lp - lm) / (2 * h)
    return d(H_FD), d(0.5 * H_FD)


@pytest.mark.parametrize("group", [0, 1, 2], ids=["hash_table", "density_mlp", "color_head"])
def test_device_gradients_against_central_differences(group):
    """Device gradients (fp16 MLPs on tcgen05, fp32 adjoint) against float64
    central differences of the oracle's loss on 86 sampled parameters per
    group (258 in all).

    Kink rule: a perturbation of +-h can cross a ReLU kink or move a ray's
    early termination, where the loss is not differentiable; an entry whose
    differences at h and h/2 disagree by more than 1e-4 (relative) is such a
    crossing and is left out.  On the smooth entries the bound is 1e-3
    relative to max(|fd|, 1e-2 * max|fd| of the group): entries two orders
    below the group's largest are held to 1e-5 of it absolutely, the scale
    at which the fp16 rounding of the forward activations (the device's
    arithmetic) sets the floor."""
    torch, d, loader, cam, pix, tgt = _case(W=24, H=24, n=64)
    _, g, _ = _gpu(torch, loader, cam, pix, tgt)
    dev = g.read()[group].astype(np.float64)
    om = orc.OracleModel(d, mimic_fp16=False)
    _, *exact, _ = om.loss_grad(cam, pix, tgt)
    nz = np.flatnonzero(exact[group])
    assert nz.size > 100
    pick = np.random.default_rng(17 + group).choice(nz, 86, replace=False)
    fd = np.array([_fd(om, cam, pix, tgt, group, int(k)) for k in pick])
    smooth = np.abs(fd[:, 0] - fd[:, 1]) <= SMOOTH * np.maximum(np.abs(fd[:, 0]), 1e-12)
    f = fd[smooth, 0]
    a = dev[pick][smooth]
    scale = np.maximum(np.abs(f), 1e-2 * np.abs(f).max())
    rel = np.abs(a - f) / scale
    cos = float(a @ f / (np.linalg.norm(a) * np.linalg.norm(f)))
    print(f"\nFD {['table', 'base', 'head'][group]}: smooth {int(smooth.sum())}/86, rel median {np.median(rel):.2e} "
          f"p95 {np.quantile(rel, 0.95):.2e} max {rel.max():.2e}, within 1e-3 {np.mean(rel <= FD_REL):.3f}, cos {cos:.7f}")
    assert smooth.sum() >= 30
    assert np.median(rel) <= FD_REL and np.quantile(rel, 0.95) <= 10 * FD_REL, rel
    assert cos > 0.99999


class RenderLoss:
    """Test-harness torch.autograd.Function over fvc_render_backward: the mean
    squared error of the plain render at `pixels` against `target`, with the
    model's parameters as differentiable inputs (table, density-MLP blob,
    color-head blob, each fp32 in the model file layout).  The renderer reads
    its parameters from the loaded model, so the tensors stand for them and
    must not be modified in place between forward and backward; target is
    differentiable too (dL/dtarget = -2/n (C + T - target))."""

    @staticmethod
    def make():
        torch = pytest.importorskip("torch")

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, table, base, head, target, renderer, network, info, pixels):
                g = fvc.Gradients(network)
                pred = torch.zeros((pixels.numel(), 4), dtype=torch.float32, device="cuda")
                loss = renderer.render_backward(info, pixels, target.detach().contiguous(), g, pred=pred)
                gt, gb, gh = (torch.from_numpy(x).to(table.device, torch.float64) for x in g.read())
                ctx.save_for_backward(gt.view_as(table), gb.view_as(base), gh.view_as(head), pred, target)
                ctx.params = (table, base, head)
                ctx.versions = tuple(t._version for t in ctx.params)
                return torch.tensor(loss, dtype=torch.float64, device=table.device)

            @staticmethod
            def backward(ctx, gout):
                gt, gb, gh, pred, target = ctx.saved_tensors
                if tuple(t._version for t in ctx.params) != ctx.versions:
                    raise RuntimeError("RenderLoss: a parameter tensor was modified in place after the forward")
                n = pred.shape[0]
                dtgt = -2.0 / n * (pred[:, :3] + pred[:, 3:4] - target)
                return gout * gt, gout * gb, gout * gh, (gout * dtgt).to(target.dtype), None, None, None, None

        return _Fn


def test_autograd_function_wrapper():
    """torch.autograd through RenderLoss: parameter gradients equal the
    library's own, agree with the float64 adjoint, and the target's gradient
    equals autograd of the loss written in torch over the returned colours."""
    torch, d, loader, cam, pix, tgt = _case(n=256)
    Fn = RenderLoss.make()
    om = orc.OracleModel(d, mimic_fp16=True)
    dev = torch.device("cuda")
    table = torch.zeros(om.table.size, dtype=torch.float64, device=dev, requires_grad=True)
    base = torch.zeros(om.base_w.size, dtype=torch.float64, device=dev, requires_grad=True)
    head = torch.zeros(om.head_w.size, dtype=torch.float64, device=dev, requires_grad=True)
    target = torch.from_numpy(tgt).to(dev).requires_grad_(True)
    r = fvc.PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    info = fvc.raymarch_info(cam, loader.stepsize_info)
    pixels = torch.from_numpy(pix).to(dev)
    loss = Fn.apply(table, base, head, target, r, loader.nerf_network, info, pixels)
    (3.0 * loss).backward()
    lref, g, pred = _gpu(torch, loader, cam, pix, tgt)
    assert abs(float(loss.detach()) - lref) <= 1e-6 * lref
    # a second call of the library: the table gradient is an atomic scatter, so its float sums may differ
    # in the last bits between calls
    for name, t, a in zip(("table", "base", "head"), (table, base, head), g.read()):
        a = 3.0 * a.astype(np.float64)
        np.testing.assert_allclose(t.grad.cpu().numpy(), a, rtol=1e-5, atol=1e-6 * np.abs(a).max(), err_msg=name)
    oloss, ot, ob, oh, _ = om.loss_grad(cam, pix, tgt)
    for name, t, b in zip(("table", "base", "head"), (table, base, head), (ot, ob, oh)):
        cos, rel = _compare(t.grad.cpu().numpy() / 3.0, b)
        assert cos > 0.9999 and rel < 2e-3, (name, cos, rel)
    # d loss / d target through autograd of the same loss written in torch
    p = torch.from_numpy(pred).to(dev)
    tt = torch.from_numpy(tgt).to(dev).requires_grad_(True)
    (3.0 * ((p[:, :3] + p[:, 3:4] - tt) ** 2).sum(1).mean()).backward()
    torch.testing.assert_close(target.grad, tt.grad, rtol=1e-5, atol=1e-7)
