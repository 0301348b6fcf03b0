"""A small, fixed rendering case for kernel profiles.

    python bench_case.py --res 960x540 --frames 2 --path plain --network tc
    python bench_case.py --res 400x400 --frames 2 --path backward --rays 65536
    python bench_case.py --res 960x540 --frames 1 --path plain --tile 256

Renders `frames` frames of the benchmark's camera path (the synthetic
3-cascade, 2^19-entry scene) at the given resolution through the C ABI and
prints one JSON line per frame: resample rows, cache rows, kernels launched
and the event-timed resample-kernel milliseconds.  The counts are
deterministic, so a run under a profiler processes exactly the rows the
plain run printed; per-row DRAM traffic is a capture's bytes divided by them.
The cached path builds its cache at frame 0 and rebuilds it whenever the
reprojected coverage drops below 0.9, like the benchmark.
"""
from __future__ import annotations

import argparse
import json
import time

from frustumvolumecaching_gb300 import camera as fcam
from frustumvolumecaching_gb300 import model as fmodel
from frustumvolumecaching_gb300.renderer import (Cache, CachePerformanceRenderer, PerformanceRenderer, default_cache_settings, load_data,
                       raymarch_info)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", default="960x540")
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--path", choices=["plain", "cached", "backward"], default="plain")
    ap.add_argument("--network", choices=["tc", "mma"], default="tc")
    ap.add_argument("--rays", type=int, default=1 << 16, help="rays per backward step")
    ap.add_argument("--tile", type=int, choices=[64, 128, 256], default=128, help="tcgen05 network tile height (plain path)")
    ap.add_argument("--batch-rows", type=int, default=0, help="compaction batch, rows per sub-iteration (0: capacity)")
    ap.add_argument("--skip", action="store_true", help="empty-space skipping in the march (off by default, as in the library)")
    ap.add_argument("--scene", choices=["c2", "c1"], default="c2",
                    help="c2: the cached workload's scene and camera path; c1: the 256x256 workload's scene, seeded camera")
    ap.add_argument("--build-tc", action="store_true", help="cache builds' density network on tcgen05 (default mma.sync)")
    ap.add_argument("--separate-classify", action="store_true",
                    help="cached path: the classification pass and two row lists instead of the classifying march")
    args = ap.parse_args(argv)
    W, H = (int(v) for v in args.res.lower().split("x"))
    if args.path == "backward":
        return backward_case(args, W, H)
    if args.scene == "c1":
        spec = fmodel.spec_config1()
        loader = load_data(fmodel.ensure_model(spec))
        cams = [fcam.seeded_camera(spec.seed, width=W, height=H)] * args.frames
    else:
        spec = fmodel.spec_config2()
        loader = load_data(fmodel.ensure_model(spec))
        cams = fcam.rotation_path(spec.seed, n_frames=args.frames, width=W, height=H)
    infos = [raymarch_info(c, loader.stepsize_info) for c in cams]
    if args.path == "plain":
        r = PerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network)
    else:
        caches = (Cache(), Cache())
        r = CachePerformanceRenderer(loader.scene_info, loader.occupancy_grid_morton_bitfield, loader.nerf_network,
                                     caches[0], caches[1])
        r.resizeCache((W, H), loader.stepsize_info)
        r.setCacheSettings(default_cache_settings())
    r.resizeRenderbuffers((W, H))
    r.set_network_path(args.network == "tc")
    r.set_tiling(args.tile, args.batch_rows)
    r.set_empty_space_skipping(args.skip)
    if args.path == "cached":
        r.set_fused_classify(not args.separate_classify)
        r.set_build_network_path(args.build_tc)
    r.set_kernel_timing(True)
    for i, info in enumerate(infos):
        build = None
        if args.path == "cached" and i == 0:
            r.initCacheBlockwise(info)
            r.swapCache()
            build = r._init_stats
        t0 = time.perf_counter()
        r.render_device(info)
        st = r._render_stats  # waits for the frame
        frame_ms = (time.perf_counter() - t0) * 1e3
        line = {"frame": i, "resample_rows": st.n_resamples, "cache_rows": st.n_cache_hits, "steps": st.n_steps,
                "launches": st.n_launches, "resample_kernel_launches": st.n_timed_launches,
                "resample_kernel_ms": round(st.timed_kernel_ms, 3), "frame_ms": round(frame_ms, 3), "guard": st.guard_flags}
        if args.path == "cached":
            cov = st.n_cache_hits / max(1, st.n_cache_hits + st.n_resamples)
            line["coverage"] = round(cov, 4)
            if cov < 0.9 and i + 1 < len(infos):
                r.initCacheBlockwise(info)
                r.swapCache()
                build = r._init_stats
            if build is not None:
                line["build_launches"] = build.n_launches
                line["bricks_demanded"] = build.n_bricks_demanded
        print(json.dumps(line), flush=True)


def backward_case(args, W: int, H: int) -> None:
    """`frames` steps of the differentiable render on the config-5 model pair:
    random rays of a WxH view against the second network's image."""
    import numpy as np
    import torch

    from frustumvolumecaching_gb300.renderer import Gradients

    spec = fmodel.spec_config5()
    train = load_data(fmodel.ensure_model(spec))
    target_net = load_data(fmodel.ensure_model(fmodel.spec_config5(target=True)))
    cam = fcam.seeded_camera(spec.seed, width=W, height=H)
    pix = np.random.default_rng(spec.seed).choice(W * H, min(args.rays, W * H), replace=False).astype(np.int32)
    tr = PerformanceRenderer(target_net.scene_info, target_net.occupancy_grid_morton_bitfield, target_net.nerf_network)
    full = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    tr.render_device(raymarch_info(cam, target_net.stepsize_info), results=full)
    tr.synchronize()
    pixels = torch.from_numpy(pix).cuda()
    flat = full.reshape(-1, 4)[pixels.long()]
    target = (flat[:, :3] + flat[:, 3:4]).contiguous()
    r = PerformanceRenderer(train.scene_info, train.occupancy_grid_morton_bitfield, train.nerf_network)
    r.set_network_path(args.network == "tc")
    g = Gradients(train.nerf_network)
    info = raymarch_info(cam, train.stepsize_info)
    for i in range(args.frames):
        loss = r.render_backward(info, pixels, target, g)
        st = r._render_stats
        print(json.dumps({"step": i, "rays": int(pix.size), "loss": loss, "samples": st.n_samples,
                          "launches": st.n_launches}), flush=True)


if __name__ == "__main__":
    main()
