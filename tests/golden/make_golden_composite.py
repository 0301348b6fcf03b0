"""Regenerates tests/golden/composite.npz from the reference's own
compositing kernel (accumulate_performance_kernel, src/performance_renderer.cu:
71-125), run on the host by oracle/_ref/ref_composite (oracle/Makefile,
target ``ref``).

Run from the repository root where the reference tree is available:
    make -C oracle ref REF=<reference checkout>
    python tests/golden/make_golden_composite.py

Two seeded batches of rays with 0..16 samples each, in the kernel's
sample-major layout: random fp16 network outputs (rgb logits, log-densities
wide enough that many rays terminate at T < 1e-4), increasing t0 on a
cone-angle step grid, some rays already finished by the march; one batch
with alpha threshold 0, one with 1e-3.
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_composite")

CONE, DT_MIN, DT_MAX = 1.0 / 256.0, 3.0 ** 0.5 / 1024.0, 0.0703125


def make_case(seed: int, n_alive: int, alpha_thre: float) -> dict:
    rng = np.random.default_rng(seed)
    smax = 16
    batch = n_alive * smax
    n_steps = rng.integers(0, smax + 1, n_alive).astype(np.int32)
    alive = (rng.uniform(size=n_alive) > 0.1).astype(np.uint8)
    res = np.zeros((n_alive, 4), np.float32)
    res[:, :3] = rng.uniform(0.0, 0.3, (n_alive, 3))
    res[:, 3] = np.where(rng.uniform(size=n_alive) < 0.5, 1.0, rng.uniform(1e-3, 1.0, n_alive))
    out = np.zeros((4, batch), np.float16)
    out[:3] = rng.normal(0.0, 2.0, (3, batch)).astype(np.float16)
    out[3] = rng.uniform(-6.0, 7.0, batch).astype(np.float16)
    t0 = np.zeros(batch, np.float32)
    t = rng.uniform(0.5, 6.0, n_alive).astype(np.float32)
    for s in range(smax):
        rows = s * n_alive + np.arange(n_alive)
        t0[rows] = t
        dt = np.clip(t * np.float32(CONE), np.float32(DT_MIN), np.float32(DT_MAX)).astype(np.float32)
        t = (t + dt * rng.integers(1, 6, n_alive).astype(np.float32)).astype(np.float32)
    return {"n_alive": n_alive, "batch": batch, "cone": CONE, "dt_min": DT_MIN, "dt_max": DT_MAX, "alpha_thre": alpha_thre,
            "n_steps": n_steps, "alive_in": alive, "results_in": res, "out4": out, "t0": t0}


def run_reference(case: dict) -> tuple[np.ndarray, np.ndarray]:
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fi, "wb") as f:
            f.write(struct.pack("<ii", case["n_alive"], case["batch"]))
            f.write(np.asarray([case["cone"], case["dt_min"], case["dt_max"], case["alpha_thre"]], np.float32).tobytes())
            f.write(case["n_steps"].astype("<i4").tobytes())
            f.write(case["alive_in"].astype(np.uint8).tobytes())
            f.write(case["results_in"].astype("<f4").tobytes())
            f.write(case["out4"].view(np.uint16).astype("<u2").tobytes())
            f.write(case["t0"].astype("<f4").tobytes())
        subprocess.run([EXE, fi, fo], check=True)
        raw = open(fo, "rb").read()
    n = case["n_alive"]
    res = np.frombuffer(raw[:16 * n], "<f4").reshape(n, 4).copy()
    alive = np.frombuffer(raw[16 * n:17 * n], np.uint8).copy()
    return res, alive


def main() -> None:
    if not os.path.exists(EXE):
        sys.exit("build oracle/_ref/ref_composite first: make -C oracle ref REF=<reference checkout>")
    out = {}
    for name, seed, thre in (("thre0", 11, 0.0), ("thre1e3", 12, 1e-3)):
        c = make_case(seed, 1024, thre)
        res, alive = run_reference(c)
        for k, v in c.items():
            out[f"{name}_{k}"] = np.asarray(v)
        out[f"{name}_results_ref"] = res
        out[f"{name}_alive_ref"] = alive
    np.savez_compressed(os.path.join(HERE, "composite.npz"), **out)
    print("wrote", os.path.join(HERE, "composite.npz"))


if __name__ == "__main__":
    main()
