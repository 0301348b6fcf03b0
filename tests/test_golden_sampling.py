"""The sampling of non-deterministic ray generation (fvc_sampling.h, shared by
the device and the oracle) against golden vectors from the reference's own
code run on the host (tests/golden/make_golden_sampling.py,
oracle/ref_sampling.cu).

Integer work is bit-exact: the Sobol points (every direction number of the
five dimensions), the scrambled values, the pixel and start-t jitter.  What
passes through sin / cos / acos (the disk map, slerp) is computed in double
precision and rounded once, where the reference calls its platform's float
functions: compared to 2 ulp of the result's scale.  Rays (origin,
direction, first t1) with motion blur and depth of field follow."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle as orc

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sampling.npz"))
EPS = np.float32(2.0 ** -23)


def test_sobol_direction_numbers_and_points_exact():
    got = np.array([orc.lib().orc_smp_sobol(int(i), int(d)) for i, d in G["sobol_in"]], np.uint32)
    np.testing.assert_array_equal(got, G["sobol_out"])


def test_scrambled_sobol_values_exact():
    got = np.array([orc.lib().orc_smp_ld_val(int(i), int(s), 0) for i, s in G["ld_in"]], np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), G["ld_out"].view(np.uint32))
    got1 = np.array([orc.lib().orc_smp_ld_val(int(i), int(s), 1) for i, s in G["ld_in"]], np.float32)
    np.testing.assert_array_equal(got1.view(np.uint32), G["ld2_out"][:, 1].copy().view(np.uint32))


def test_pixel_and_t_jitter_exact():
    out = np.zeros(2, np.float32)
    for spp, ref in zip(G["spp_in"], G["spp_out"]):
        orc.lib().orc_smp_pixel_offset(int(spp), orc.ptr(out))
        np.testing.assert_array_equal(out.view(np.uint32), ref.view(np.uint32))
    got = np.array([orc.lib().orc_smp_t_offset(int(s), int(r)) for s, r in G["toff_in"]], np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), G["toff_out"].view(np.uint32))
    assert len(set(G["spp_out"][:, 0].tolist())) == 256  # 256 distinct sub-pixel positions


def test_square_to_disk_close():
    out = np.zeros(2, np.float32)
    got = []
    for a, b in G["disk_in"]:
        orc.lib().orc_smp_square_to_disk(float(a), float(b), orc.ptr(out))
        got.append(out.copy())
    got = np.asarray(got)
    ref = G["disk_out"]
    ok = np.isfinite(ref)
    np.testing.assert_array_equal(np.isfinite(got), ok)
    assert np.abs(got[ok] - ref[ok]).max() <= 2 * EPS
    assert np.mean(got[ok] == ref[ok]) > 0.9
    assert np.all(np.hypot(got[:, 0], got[:, 1]) <= 1.0 + 4 * EPS)


def test_camera_slerp_close():
    out = np.zeros(12, np.float32)
    got = []
    for row in G["slerp_in"]:
        a = np.ascontiguousarray(row[:12])
        b = np.ascontiguousarray(row[12:24])
        orc.lib().orc_smp_camera_slerp(orc.ptr(a), orc.ptr(b), float(row[24]), orc.ptr(out))
        got.append(out.copy())
    got = np.asarray(got)
    ref = G["slerp_out"]
    rot = np.r_[0:3, 4:7, 8:11]
    assert np.abs(got[:, rot] - ref[:, rot]).max() <= 8 * EPS
    np.testing.assert_array_equal(got[:, [3, 7, 11]], ref[:, [3, 7, 11]])  # translation: plain float arithmetic


def _cam():
    W, H = (int(v) for v in G["cam_res"])
    fx, fy, px, py = (float(v) for v in G["cam_intr"])
    c2w = G["cam_c2w"].astype(np.float64)
    return {"resolution": (W, H), "is_open_gl": False, "focal": (fx, fy), "principal": (px, py),
            "cam2world": c2w, "world2cam": np.zeros((3, 4)), "deterministic": False,
            "next_cam2world": G["cam_next"], "aperature": float(G["cam_lens"][0]), "focus_z": float(G["cam_lens"][1])}


@pytest.mark.parametrize("flags", [0, 1, 2, 3], ids=["jitter", "motion_blur", "depth_of_field", "both"])
def test_generated_rays_against_reference(flags):
    """Origin, direction and first t1 of non-deterministic rays: exact with
    jitter only (no transcendental); within a few ulp of the scene scale with
    motion blur or depth of field."""
    s = G["scene"]
    scene = orc.OrcScene()
    scene.grid_nlvl = int(G["scene_nlvl"])
    scene.contraction = 1
    scene.aabb_from[:], scene.aabb_to[:] = s[:3].tolist(), s[3:6].tolist()
    scene.c_from[:], scene.c_to[:] = s[:3].tolist(), s[3:6].tolist()
    steps = orc.make_steps(scene, float(s[6]), float(s[7]), float(s[8]), float(s[9]), True)
    out = np.zeros(8, np.float32)
    rows = np.flatnonzero(G["rays_in"][:, 3] == flags)
    assert rows.size > 50
    worst = 0.0
    for i in rows:
        x, y, spp, fl = (int(v) for v in G["rays_in"][i])
        cam = dict(_cam(), sample_index=spp, motion_blur=bool(fl & 1))
        if not fl & 2:
            cam["aperature"] = 0.0
        orc.lib().orc_generate_ray(C.byref(scene), C.byref(steps), C.byref(orc.make_cam(cam)), x, y, orc.ptr(out))
        ref = G["rays_out"][i]
        assert out[7] == ref[7]
        if flags == 0:
            np.testing.assert_array_equal(out.view(np.uint32), ref.view(np.uint32))
        else:
            worst = max(worst, float(np.abs(out[:6] - ref[:6]).max()))
            if ref[7]:
                assert abs(out[6] - ref[6]) <= 1e-4 * max(1.0, abs(ref[6])), (out, ref)
    assert worst <= 2e-6, worst
