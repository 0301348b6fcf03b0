"""Host side of the view-dependent split network: the model export carries
mlp_first_head in the layout NerfNetwork::init_viewdep reads
(include/nerf_network.h:120-158, src/loader.cu:251-262), and the oracle
evaluates it (first head on the initial direction, SH-difference head input)."""
import json
import os

import numpy as np

from frustumvolumecaching_gb300 import model as fmodel
from oracle import oracle as orc
from tests.helpers import small_camera


def _vd_spec():
    spec = fmodel.spec_tiny(seed=31)
    spec.view_dependent = True
    spec.name = f"{spec.name}_h2"
    return spec


def test_export_layout():
    d = fmodel.ensure_model(_vd_spec())
    cfg = json.load(open(os.path.join(d, "config.json")))
    fh = cfg["mlp_first_head"]
    assert fh["n_input"] == 32 and fh["n_output"] == 8 and fh["network"]["n_hidden_layers"] == 1
    assert cfg["mlp_head"]["n_input"] == 8 + 16 + 16
    assert os.path.getsize(os.path.join(d, "mlp_first_head.dat")) == (64 * 32 + 16 * 64) * 2
    assert os.path.getsize(os.path.join(d, "mlp_head.dat")) == (64 * 48 + 64 * 64 + 16 * 64) * 2


def test_oracle_renders_the_split_network():
    vd = orc.OracleModel(fmodel.ensure_model(_vd_spec()), mimic_fp16=True)
    plain_spec = fmodel.spec_tiny(seed=31)
    plain = orc.OracleModel(fmodel.ensure_model(plain_spec), mimic_fp16=True)
    cam = small_camera(1001, 24, 16)
    a, ns_a, _ = vd.render_plain(cam)
    b, ns_b, _ = plain.render_plain(cam)
    assert np.isfinite(a).all()
    np.testing.assert_array_equal(ns_a, ns_b)  # the density network and the occupancy are the same
    assert np.abs(a - b).max() > 1e-3           # the colours come from the split head
