"""The oracle's compositing against the reference's own compositing kernel.

tests/golden/composite.npz holds two batches of rays (network outputs, t0,
incoming ray results) and what accumulate_performance_kernel
(src/performance_renderer.cu:71-125), compiled from the reference tree and run
on the host (oracle/ref_composite.cu, tests/golden/make_golden_composite.py),
made of them.  The oracle composites the same rows in float64: the
termination (alive flags) must be identical and rgb / T within 2e-6 of the
kernel's float32 sums.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "composite.npz")


@pytest.mark.parametrize("name", ["thre0", "thre1e3"])
def test_oracle_composites_like_the_reference_kernel(name):
    g = np.load(GOLDEN)
    v = {k[len(name) + 1:]: g[k] for k in g.files if k.startswith(name + "_")}
    n, batch = int(v["n_alive"]), int(v["batch"])
    steps = orc.OrcSteps()
    steps.cone_angle, steps.dt_min, steps.dt_max = float(v["cone"]), float(v["dt_min"]), float(v["dt_max"])
    res = v["results_in"].astype(np.float32).copy()
    alive = v["alive_in"].astype(np.uint8).copy()
    out4 = v["out4"].astype(np.float32)
    t0 = v["t0"].astype(np.float32)
    n_steps = v["n_steps"].astype(np.int32)
    orc.lib().orc_composite_rows(n, batch, orc.C.byref(steps), float(v["alpha_thre"]), orc.ptr(n_steps), orc.ptr(alive),
                                 orc.ptr(res), orc.ptr(out4), orc.ptr(t0))
    np.testing.assert_array_equal(alive, v["alive_ref"])
    err = np.abs(res - v["results_ref"]).max()
    terminated = int((v["alive_in"] == 1).sum() - (alive == 1).sum())
    print(f"\n{name}: {n} rays, {int(n_steps.sum())} samples, {terminated} terminated here, max-abs vs reference {err:.2e}")
    assert terminated > 50
    assert err <= 2e-6, err
