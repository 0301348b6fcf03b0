"""C-ABI library checks that need no GPU: it loads, exports every entry
point include/fvc.h declares, and reports loader errors with status codes."""
import json
import os
import re
import shutil

import numpy as np
import pytest

from frustumvolumecaching_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "fvc.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fvc_[a-z0-9_]+)\s*\(", txt)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = L.load()
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/fvc.h but not exported"
    assert set(syms) <= set(L.SIGNATURES), set(syms) - set(L.SIGNATURES)
    assert lib.fvc_version().decode().startswith("fvc-gb300")


def test_struct_layouts_match_reference():
    import ctypes as C
    assert C.sizeof(L.SceneInfo) == 76
    assert L.SceneInfo.aabb_from.offset == 16 and L.SceneInfo.alpha_thre.offset == 72
    assert C.sizeof(L.StepsizeInfo) == 48
    assert C.sizeof(L.CameraInfo) == 144 and L.CameraInfo.focal.offset == 16 and L.CameraInfo.focus_z.offset == 132
    assert C.sizeof(L.RaymarchInfo) == 352 and L.RaymarchInfo.deterministic.offset == 341
    assert C.sizeof(L.RayResult) == 16


def _load(path):
    import ctypes as C
    h = C.c_void_p()
    rc = L.load().fvc_model_load(path.encode(), C.byref(h))
    return rc, L.load().fvc_last_error().decode()


def test_loader_missing_directory(tmp_path):
    rc, msg = _load(str(tmp_path / "nope"))
    assert rc == 7 and "config" in msg


def test_loader_malformed_config(tmp_path):
    (tmp_path / "config.json").write_text("{ not json")
    rc, msg = _load(str(tmp_path))
    assert rc == 2


def test_loader_rejects_unsupported_grid(tmp_path):
    from tests.helpers import tiny_model
    src = tiny_model()
    d = tmp_path / "m"
    shutil.copytree(src, d)
    cfg = json.load(open(d / "config.json"))
    cfg["scene"]["grid_resolution"] = 64
    json.dump(cfg, open(d / "config.json", "w"))
    rc, msg = _load(str(d))
    assert rc == 2 and "grid resolution" in msg


def test_loader_truncated_table(tmp_path):
    from tests.helpers import tiny_model
    src = tiny_model()
    d = tmp_path / "m"
    shutil.copytree(src, d)
    data = open(d / "pos_enc.dat", "rb").read()
    open(d / "pos_enc.dat", "wb").write(data[:-2])
    rc, msg = _load(str(d))
    assert rc == 7 and "pos_enc.dat" in msg


def test_null_arguments_are_rejected():
    import ctypes as C
    lib = L.load()
    assert lib.fvc_model_load(None, None) == 6
    assert lib.fvc_renderer_resize(None, 4, 4) == 6
    assert lib.fvc_render(None, None, None) == 6


@pytest.mark.parametrize("aabb,cone,step,near", [((-1.5, 1.5), 0.0, 3 / 1024, 0.0), ((-6.0, 6.0), 1 / 256, 3 ** 0.5 / 1024, 0.0),
                                                  ((-6.0, 6.0), 1 / 512, 3 ** 0.5 / 2048, 0.2), ((-2.0, 3.0), 1 / 256, 0.004, 0.05)])
def test_stepsize_setup_matches_the_oracle(aabb, cone, step, near):
    """fvc_stepsize_setup (StepsizeInfo::setAdditionalInfo, host only) fills
    the same derived fields as the oracle's restatement, bit for bit; and
    change_sampling_rate(2) equals a setup at half the cone and step."""
    import ctypes as C
    from frustumvolumecaching_gb300.renderer import change_sampling_rate
    from oracle import oracle as orc
    sc = L.SceneInfo()
    sc.grid_resolution, sc.grid_nlvl = 128, 1
    for f in ("x", "y", "z"):
        setattr(sc.aabb_from, f, aabb[0])
        setattr(sc.aabb_to, f, aabb[1])
    st = L.StepsizeInfo()
    st.cone_angle, st.stepsize, st.near, st.far = cone, step, near, 1e10
    L.check(L.load().fvc_stepsize_setup(C.byref(sc), C.byref(st)))
    osc = orc.make_scene({"grid_nlvl": 1, "aabb": [aabb[0]] * 3 + [aabb[1]] * 3, "alpha_thre": 0.0})
    ost = orc.make_steps(osc, cone, step, near, 1e10)
    names = ["dt_min", "dt_max", "t_min", "t_max", "i_min", "i_max", "near_i"] + (["log1p_c"] if cone > 0 else [])
    for n in names:
        a, b = np.float32(getattr(st, n)), np.float32(getattr(ost, "near_i" if n == "near_i" else n))
        assert a.view(np.uint32) == b.view(np.uint32), (n, a, b)
    half = change_sampling_rate(st, 2.0, sc)
    ref = orc.make_steps(osc, np.float32(cone) / np.float32(2), np.float32(step) / np.float32(2), near, 1e10)
    for n in names:
        a, b = np.float32(getattr(half, n)), np.float32(getattr(ref, n))
        assert a.view(np.uint32) == b.view(np.uint32), (n, a, b)
