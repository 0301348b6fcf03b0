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
