"""The CPU oracle's marcher against golden vectors made by the reference's own
header math (tests/golden/make_golden.py, oracle/ref_golden.cu)."""
import ctypes as C
import os
import zlib

import numpy as np
import pytest

from oracle import oracle as orc
from tests.golden.golden_scenes import SCENES, occupancy_grid, pixels, points

HERE = os.path.dirname(os.path.abspath(__file__))


def _setup(name, use_libm):
    sc = SCENES[name]
    g = np.load(os.path.join(HERE, "golden", f"march_{name}.npz"))
    scene = orc.OrcScene()
    scene.grid_nlvl = sc["nlvl"]
    scene.contraction = 3 if sc["contraction"] else 1
    scene.aabb_from[:], scene.aabb_to[:] = sc["aabb"][:3], sc["aabb"][3:]
    scene.c_from[:], scene.c_to[:] = sc["caabb"][:3], sc["caabb"][3:]
    steps = orc.make_steps(scene, sc["cone"], sc["stepsize"], sc["near"], sc["far"], use_libm)
    cam = orc.OrcCam()
    cam.W, cam.H, cam.fx, cam.fy, cam.px, cam.py = sc["W"], sc["H"], sc["fx"], sc["fy"], sc["px"], sc["py"]
    cam.c2w[:] = np.asarray(sc["c2w"], np.float32).tolist()
    grid = occupancy_grid(sc["nlvl"])
    bits = np.zeros(grid.size // 8, np.uint8)
    orc.lib().orc_grid_to_morton_bits(orc.ptr(grid), sc["nlvl"], orc.ptr(bits))
    return sc, g, scene, steps, cam, bits


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_step_setup_matches_reference(name):
    sc, g, scene, steps, cam, bits = _setup(name, True)
    mine = np.asarray([steps.dt_min, steps.dt_max, steps.t_min, steps.t_max, steps.i_min, steps.i_max,
                       steps.log1p_c, steps.near_i], np.float32)
    np.testing.assert_array_equal(mine.view(np.uint32), g["steps"].view(np.uint32))


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_traces_bit_exact_with_reference_libm(name):
    """With the host libm log/pow the oracle reproduces every ray's start,
    far, step sequence and occupancy bits of the reference header."""
    sc, g, scene, steps, cam, bits = _setup(name, True)
    _check_traces(sc, g, scene, steps, cam, bits, exact=True)


def test_traces_c1_deterministic_math_identical():
    """cone_angle = 0: no transcendental in the index math, so the
    deterministic build is bit-exact with the reference too."""
    sc, g, scene, steps, cam, bits = _setup("c1", False)
    _check_traces(sc, g, scene, steps, cam, bits, exact=True)


def test_traces_c2_deterministic_math_close():
    """cone_angle > 0: the kernels use fvc_detmath log/exp (host==device)
    instead of libm; the step grid may move by a few ulp, which changes at
    most a tiny fraction of occupancy decisions."""
    sc, g, scene, steps, cam, bits = _setup("c2", False)
    stats = _check_traces(sc, g, scene, steps, cam, bits, exact=False)
    assert stats["ray_mismatch"] <= 0.02 * stats["rays"], stats


def _check_traces(sc, g, scene, steps, cam, bits, exact):
    pix = pixels(sc)
    max_steps = sc["max_steps"]
    t0b = np.zeros(max_steps, np.uint32)
    occ = np.zeros(max_steps, np.uint8)
    init = np.zeros(3, np.float32)
    mism = 0
    for i, (x, y) in enumerate(pix):
        n = orc.lib().orc_trace_ray(C.byref(scene), C.byref(steps), C.byref(cam), orc.ptr(bits), int(x), int(y),
                                    max_steps, orc.ptr(t0b), orc.ptr(occ), orc.ptr(init))
        assert int(init[2]) == g["hits"][i]
        if exact:
            assert init[0].view(np.uint32) == g["start"][i].view(np.uint32), (i, init[0], g["start"][i])
            assert init[1].view(np.uint32) == g["far"][i].view(np.uint32)
            assert n == g["n_steps"][i], (i, n, g["n_steps"][i])
            t0 = t0b[:n].view(np.float32)
            crc = zlib.crc32(t0.tobytes()) ^ (zlib.crc32(occ[:n].tobytes()) << 1 & 0xFFFFFFFF)
            assert crc == int(g["crc"][i]), i
            a, b = g["occ_off"][i], g["occ_off"][i + 1]
            np.testing.assert_array_equal(np.nonzero(occ[:n])[0], g["occ_steps"][a:b])
        else:
            a, b = g["occ_off"][i], g["occ_off"][i + 1]
            if n != g["n_steps"][i] or not np.array_equal(np.nonzero(occ[:n])[0], g["occ_steps"][a:b]):
                mism += 1
    return {"rays": len(pix), "ray_mismatch": mism}


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_point_functions(name):
    sc, g, scene, steps, cam, bits = _setup(name, True)
    pts = points(sc)
    for i, p in enumerate(pts):
        a = np.float32(abs(p[0]) * np.float32(4.0) + np.float32(0.001))
        assert np.float32(orc.lib().orc_step_from_t(C.byref(steps), a)).view(np.uint32) == g["pt_step_from_t"][i].view(np.uint32)
        assert np.float32(orc.lib().orc_t_from_step(C.byref(steps), np.float32(a * np.float32(100.0)))).view(np.uint32) == \
            g["pt_t_from_step"][i].view(np.uint32)
        out = np.zeros(3, np.float32)
        orc.lib().orc_contract(C.byref(scene), orc.ptr(np.ascontiguousarray(p)), orc.ptr(out))
        np.testing.assert_array_equal(out.view(np.uint32), g["pt_contract"][i].view(np.uint32))
        cell = np.zeros(1, np.int32)
        assert orc.lib().orc_occupied(C.byref(scene), orc.ptr(bits), orc.ptr(np.ascontiguousarray(p)), orc.ptr(cell)) == g["pt_occ"][i]
