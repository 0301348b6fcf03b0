"""The kernels' exact division by a known denominator (div_rn_by: the
correctly rounded reciprocal and Markstein's one-step correction) against
the hardware IEEE division and numpy's float32 division, bit for bit, on
random operands over 2^-60..2^60 with quotients in 2^-100..2^100, on the
scene extents the marcher divides by, and on the per-ray denominators
(camera-space depths, contraction norms)."""
import numpy as np
import pytest


from frustumvolumecaching_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _run(x, d):
    x = np.ascontiguousarray(x, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    q = np.zeros_like(x)
    qi = np.zeros_like(x)
    L.check(L.load().fvc_selftest_division(L.ptr(x), L.ptr(d), x.size, L.ptr(q), L.ptr(qi)))
    return q, qi, (x / d).astype(np.float32)


def test_random_operands_bit_exact():
    rng = np.random.default_rng(21)
    n = 1 << 22
    x = (np.exp2(rng.uniform(-60, 60, n)) * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    d = (np.exp2(rng.uniform(-60, 60, n)) * rng.choice([-1.0, 1.0], n)).astype(np.float32)
    ok = np.abs(np.log2(np.abs(x.astype(np.float64) / d))) < 100
    q, qi, ref = _run(x[ok], d[ok])
    np.testing.assert_array_equal(q.view(np.uint32), qi.view(np.uint32))
    np.testing.assert_array_equal(q.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("den", [3.0, 12.0, 0.75, 1.5, 6.0, 3.0 / 4.0, 12.0 / 4.0, 1.0 / 3.0, 2.0, 0.1, 7.3])
def test_scene_denominators_bit_exact(den):
    rng = np.random.default_rng(int(den * 1000))
    x = rng.uniform(-24.0, 24.0, 1 << 20).astype(np.float32)
    x[:4] = [0.0, 1.0, -1.0, den]
    q, qi, ref = _run(x, np.full_like(x, den))
    np.testing.assert_array_equal(q.view(np.uint32)[4:], ref.view(np.uint32)[4:])
    np.testing.assert_array_equal(q[:4], ref[:4])  # signed zeros compare equal
    np.testing.assert_array_equal(qi.view(np.uint32), ref.view(np.uint32))



def test_per_ray_denominators_bit_exact():
    """x / z of the froxel projection and u / f of the L-inf contraction:
    both operands vary (z in 1e-3..1e3, f in 1..2^10)."""
    rng = np.random.default_rng(22)
    n = 1 << 21
    z = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), n)).astype(np.float32) * rng.choice([-1.0, 1.0], n).astype(np.float32)
    x = rng.uniform(-50, 50, n).astype(np.float32)
    q, _, ref = _run(x, z)
    np.testing.assert_array_equal(q.view(np.uint32), ref.view(np.uint32))
    f = np.exp2(rng.uniform(0, 10, n)).astype(np.float32)
    u = (rng.uniform(-1, 1, n) * f).astype(np.float32)
    q, _, ref = _run(u, f)
    np.testing.assert_array_equal(q.view(np.uint32), ref.view(np.uint32))
