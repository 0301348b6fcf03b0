/*
 * fvc_sampling.h - the non-deterministic ray generation's sampling, written
 * once for the device and the host (the oracle includes it), with IEEE
 * float operations in a fixed order and no fused multiply-add, so both sides
 * give the same bits.
 *
 * What it restates (RaymarchInfo::deterministic = false):
 *   - pixel jitter and start-t jitter: ld_random_pixel_offset /
 *     ld_random_t_offset (include/util/random_val.h:320-331), a shuffled,
 *     Owen-scrambled Sobol sequence;
 *   - depth of field: square2disk_shirley (:108-127), the concentric map of
 *     Shirley and Chiu, "A Low Distortion Map Between Disk and Square"
 *     (JGT 1997);
 *   - motion blur: camera_slerp (include/raymarch_common.h:203-216) over
 *     quaternions (include/util/quat.h): Shoemake's slerp ("Animating
 *     Rotation with Quaternion Curves", SIGGRAPH 1985).
 *
 * Sobol: the first five dimensions of Joe and Kuo's direction numbers
 * ("Constructing Sobol sequences with better two-dimensional projections",
 * SIAM J. Sci. Comput. 2008; dimension 0 is the van der Corput sequence),
 * generated here from their primitive polynomials and initial numbers by the
 * Bratley-Fox recurrence instead of a table.  Scrambling: Burley,
 * "Practical Hash-based Owen Scrambling" (JCGT 9(4), 2020) - the
 * Laine-Karras style permutation on the bit-reversed value with that paper's
 * multipliers, and the index shuffled by the same nested scramble.  The seed
 * of dimension d is hash_combine(seed, d) = seed ^ (d + (seed << 6) +
 * (seed >> 2)).  A 32-bit value v becomes the float (float)v * 2^-32.
 *
 * Transcendentals (the disk map's sin/cos, slerp's acos and sin) are
 * evaluated in double precision by the series below and rounded once to
 * float; the reference calls sincosf / acos / sin of its platform, whose
 * float results agree with a correctly rounded value to an ulp or so.
 */
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define SMP_HD __host__ __device__ __forceinline__
#else
#define SMP_HD inline
#endif

#if defined(__CUDA_ARCH__)
#define SMP_FADD(a, b) __fadd_rn((a), (b))
#define SMP_FSUB(a, b) __fsub_rn((a), (b))
#define SMP_FMUL(a, b) __fmul_rn((a), (b))
#define SMP_FDIV(a, b) __fdiv_rn((a), (b))
#define SMP_FSQRT(a) __fsqrt_rn(a)
#define SMP_DADD(a, b) __dadd_rn((a), (b))
#define SMP_DSUB(a, b) __dsub_rn((a), (b))
#define SMP_DMUL(a, b) __dmul_rn((a), (b))
#define SMP_DDIV(a, b) __ddiv_rn((a), (b))
#define SMP_DSQRT(a) __dsqrt_rn(a)
#define SMP_U2F(v) __uint2float_rn(v)
#else
#include <cmath>
/* the host side compiles with -ffp-contract=off: each operator is one IEEE operation */
#define SMP_FADD(a, b) ((a) + (b))
#define SMP_FSUB(a, b) ((a) - (b))
#define SMP_FMUL(a, b) ((a) * (b))
#define SMP_FDIV(a, b) ((a) / (b))
#define SMP_FSQRT(a) std::sqrt((float)(a))
#define SMP_DADD(a, b) ((a) + (b))
#define SMP_DSUB(a, b) ((a) - (b))
#define SMP_DMUL(a, b) ((a) * (b))
#define SMP_DDIV(a, b) ((a) / (b))
#define SMP_DSQRT(a) std::sqrt((double)(a))
#define SMP_U2F(v) ((float)(uint32_t)(v))
#endif

namespace fvc_smp {

constexpr float PI_F = 3.14159265358979323846f;

/* ---------------------------------------------------------------- Sobol */

/* primitive polynomial degree s, its interior coefficients a (s-1 bits, the
 * first coefficient in the highest bit) and the initial direction numbers
 * m_1..m_s of Sobol dimensions 1..4 (Joe-Kuo dimensions 2..5) */
struct SobolPoly { uint32_t s, a, m[3]; };

SMP_HD SobolPoly sobol_poly(uint32_t dim)
{
    switch (dim) {
    case 1: return {1u, 0u, {1u, 0u, 0u}};
    case 2: return {2u, 1u, {1u, 3u, 0u}};
    case 3: return {3u, 1u, {1u, 3u, 1u}};
    default: return {3u, 2u, {1u, 1u, 1u}};
    }
}

/* component `dim` (0..4) of Sobol point `index` as a 32-bit fraction:
 * the xor of the direction numbers v_k = m_k 2^(31-k) of the index's set bits,
 * m_k for k >= s from m_k = (xor_j 2^j a_j m_{k-j}, j = 1..s-1) ^ 2^s m_{k-s} ^ m_{k-s} */
SMP_HD uint32_t sobol(uint32_t index, uint32_t dim)
{
    if (dim == 0) {
        uint32_t x = 0u;
        for (uint32_t k = 0; k < 32; ++k)
            if ((index >> k) & 1u) x ^= 1u << (31 - k);
        return x;
    }
    const SobolPoly P = sobol_poly(dim);
    uint32_t m[32];
    uint32_t x = 0u;
    for (uint32_t k = 0; k < 32; ++k) {
        uint32_t mk;
        if (k < P.s) {
            mk = P.m[k];
        } else {
            mk = (m[k - P.s] << P.s) ^ m[k - P.s];
            for (uint32_t j = 1; j < P.s; ++j)
                if ((P.a >> (P.s - 1 - j)) & 1u) mk ^= m[k - j] << j;
        }
        m[k] = mk;
        if ((index >> k) & 1u) x ^= mk << (31 - k);
    }
    return x;
}

SMP_HD uint32_t reverse_bits(uint32_t x)
{
    uint32_t r = 0u;
    for (int k = 0; k < 32; ++k) r |= ((x >> k) & 1u) << (31 - k);
    return r;
}

SMP_HD uint32_t hash_combine(uint32_t seed, uint32_t v) { return seed ^ (v + (seed << 6) + (seed >> 2)); }

/* Burley's hash-based Owen scramble of a base-2 digit string: a
 * Laine-Karras style permutation applied to the bit-reversed value */
SMP_HD uint32_t owen_scramble(uint32_t x, uint32_t seed)
{
    x = reverse_bits(x);
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return reverse_bits(x);
}

SMP_HD float u32_to_unit(uint32_t v) { return SMP_FMUL(SMP_U2F(v), 2.3283064365386963e-10f); /* 2^-32 */ }

/* one component of the shuffled scrambled Sobol point (ld_random_val) */
SMP_HD float ld_val(uint32_t index, uint32_t seed, uint32_t dim = 0)
{
    const uint32_t i = owen_scramble(index, seed);
    return u32_to_unit(owen_scramble(sobol(i, dim), hash_combine(seed, dim)));
}

/* two components of one shuffled scrambled Sobol point (ld_random_val_2d) */
SMP_HD void ld_val2(uint32_t index, uint32_t seed, float &a, float &b)
{
    const uint32_t i = owen_scramble(index, seed);
    a = u32_to_unit(owen_scramble(sobol(i, 0), hash_combine(seed, 0)));
    b = u32_to_unit(owen_scramble(sobol(i, 1), hash_combine(seed, 1)));
}

SMP_HD float fract(float x)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(x, floorf(x));
#else
    return x - std::floor(x);
#endif
}

constexpr uint32_t PIXEL_SEED = 0xdeadbeefu;

/* ld_random_pixel_offset(sample_index): the sub-pixel position of every pixel's ray */
SMP_HD void pixel_offset(uint32_t spp, float &ox, float &oy)
{
    float a, b;
    ld_val2(spp, PIXEL_SEED, a, b);
    ox = fract(a);
    oy = fract(b);
}

/* ld_random_t_offset(sample_index, ray_id * 56924617): the start jitter in units of the first step */
SMP_HD float t_offset(uint32_t spp, uint32_t ray_id) { return fract(ld_val(spp, ray_id * 56924617u)); }

/* ------------------------------------------------- double-precision series */

/* sin and cos of x for |x| <= pi/4 (Taylor series to x^25 / x^24: the
 * truncation stays below 2^-60 relative) */
SMP_HD double sin_small(double x)
{
    const double x2 = SMP_DMUL(x, x);
    double term = x, sum = x;
    for (int k = 1; k <= 12; ++k) {
        term = SMP_DDIV(SMP_DMUL(-term, x2), (double)((2 * k) * (2 * k + 1)));
        sum = SMP_DADD(sum, term);
    }
    return sum;
}
SMP_HD double cos_small(double x)
{
    const double x2 = SMP_DMUL(x, x);
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 12; ++k) {
        term = SMP_DDIV(SMP_DMUL(-term, x2), (double)((2 * k - 1) * (2 * k)));
        sum = SMP_DADD(sum, term);
    }
    return sum;
}

/* sin and cos of a float argument of moderate size (|x| < 2^20): x - q pi/2
 * with pi/2 as its double rounding plus the remainder (6.1e-17), then the
 * series by quadrant.  The reduction loses a few double ulps at most, far
 * below the float result's rounding. */
SMP_HD void sincos_d(float xf, double &s, double &c)
{
    const double x = (double)xf;
    const double PIO2_HI = 1.5707963267948966, PIO2_LO = 6.123233995736766e-17;
    const double qd = SMP_DMUL(x, 0.6366197723675814); /* 2 / pi */
    const double q = (double)(long long)(qd < 0.0 ? SMP_DSUB(qd, 0.5) : SMP_DADD(qd, 0.5));
    double r = SMP_DSUB(x, SMP_DMUL(q, PIO2_HI));
    r = SMP_DSUB(r, SMP_DMUL(q, PIO2_LO));
    const double sr = sin_small(r), cr = cos_small(r);
    const int quad = (int)(((long long)q) & 3);
    switch (quad) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
    }
}

SMP_HD float sinf_d(float x) { double s, c; sincos_d(x, s, c); return (float)s; }

/* asin(y) for |y| <= 0.5 by its Maclaurin series (the term ratio stays below
 * y^2 (2k-1)^2 / (2k (2k+1)) < 0.25: 26 terms) */
SMP_HD double asin_small(double y)
{
    const double y2 = SMP_DMUL(y, y);
    double term = y, sum = y;
    for (int k = 1; k <= 26; ++k) {
        term = SMP_DMUL(term, SMP_DDIV(SMP_DMUL(y2, (double)((2 * k - 1) * (2 * k - 1))), (double)((2 * k) * (2 * k + 1))));
        sum = SMP_DADD(sum, term);
    }
    return sum;
}

/* acos of a float in [-1, 1]: pi/2 - asin(x) for |x| <= 1/2, else
 * 2 asin(sqrt((1 - |x|) / 2)) reflected for negative x */
SMP_HD float acosf_d(float xf)
{
    const double PI_D = 3.141592653589793, HALF_PI = 1.5707963267948966;
    const double x = (double)xf;
    double r;
    if (x >= -0.5 && x <= 0.5) {
        r = SMP_DSUB(HALF_PI, asin_small(x));
    } else {
        const double ax = x < 0.0 ? -x : x;
        const double h = SMP_DMUL(2.0, asin_small(SMP_DSQRT(SMP_DMUL(SMP_DSUB(1.0, ax), 0.5))));
        r = x < 0.0 ? SMP_DSUB(PI_D, h) : h;
    }
    return (float)r;
}

/* ---------------------------------------------------- depth of field */

/* square2disk_shirley: (a, b) in [-1, 1]^2 to the unit disk */
SMP_HD void square_to_disk(float a, float b, float &x, float &y)
{
    float r, phi;
    if (SMP_FMUL(a, a) > SMP_FMUL(b, b)) {
        r = a;
        phi = SMP_FMUL(SMP_FDIV(PI_F, 4.0f), SMP_FDIV(b, a));
    } else {
        r = b;
        phi = SMP_FSUB(SMP_FDIV(PI_F, 2.0f), SMP_FMUL(SMP_FDIV(PI_F, 4.0f), SMP_FDIV(a, b)));
    }
    double s, c;
    sincos_d(phi, s, c);
    x = SMP_FMUL(r, (float)c);
    y = SMP_FMUL(r, (float)s);
}

/* the lens offset of a pixel's ray: aperature * disk(2 u - 1) with u the 2-D
 * point seeded by the pixel (screen point scaled by the resolution, as
 * generateRay does, include/raymarch_common.h:236-239) */
SMP_HD void lens_offset(uint32_t spp, float sx, float sy, int W, int H, float aperature, float &bx, float &by)
{
    const int px = (int)SMP_FMUL(sx, (float)W), py = (int)SMP_FMUL(sy, (float)H);
    float u, v;
    ld_val2(spp, (uint32_t)px * 19349663u + (uint32_t)py * 96925573u, u, v);
    float dx, dy;
    square_to_disk(SMP_FSUB(SMP_FMUL(u, 2.0f), 1.0f), SMP_FSUB(SMP_FMUL(v, 2.0f), 1.0f), dx, dy);
    bx = SMP_FMUL(aperature, dx);
    by = SMP_FMUL(aperature, dy);
}

/* ------------------------------------------------------- motion blur */

struct Quat { float w, x, y, z; };

/* the rotation of a row-major 3x4 camera matrix as a quaternion (the
 * branch on the trace and the largest diagonal term, include/util/quat.h:10-38) */
SMP_HD Quat quat_from(const float *m)
{
    const float m00 = m[0], m01 = m[1], m02 = m[2], m10 = m[4], m11 = m[5], m12 = m[6], m20 = m[8], m21 = m[9], m22 = m[10];
    const float tr = SMP_FADD(SMP_FADD(m00, m11), m22);
    Quat q;
    if (tr > 0.0f) {
        const float S = SMP_FMUL(SMP_FSQRT(SMP_FADD(tr, 1.0f)), 2.0f);
        q.w = SMP_FMUL(0.25f, S);
        q.x = SMP_FDIV(SMP_FSUB(m21, m12), S);
        q.y = SMP_FDIV(SMP_FSUB(m02, m20), S);
        q.z = SMP_FDIV(SMP_FSUB(m10, m01), S);
    } else if (m00 > m11 && m00 > m22) {
        const float S = SMP_FMUL(SMP_FSQRT(SMP_FSUB(SMP_FSUB(SMP_FADD(1.0f, m00), m11), m22)), 2.0f);
        q.w = SMP_FDIV(SMP_FSUB(m21, m12), S);
        q.x = SMP_FMUL(0.25f, S);
        q.y = SMP_FDIV(SMP_FADD(m01, m10), S);
        q.z = SMP_FDIV(SMP_FADD(m02, m20), S);
    } else if (m11 > m22) {
        const float S = SMP_FMUL(SMP_FSQRT(SMP_FSUB(SMP_FSUB(SMP_FADD(1.0f, m11), m00), m22)), 2.0f);
        q.w = SMP_FDIV(SMP_FSUB(m02, m20), S);
        q.x = SMP_FDIV(SMP_FADD(m01, m10), S);
        q.y = SMP_FMUL(0.25f, S);
        q.z = SMP_FDIV(SMP_FADD(m12, m21), S);
    } else {
        const float S = SMP_FMUL(SMP_FSQRT(SMP_FSUB(SMP_FSUB(SMP_FADD(1.0f, m22), m00), m11)), 2.0f);
        q.w = SMP_FDIV(SMP_FSUB(m10, m01), S);
        q.x = SMP_FDIV(SMP_FADD(m02, m20), S);
        q.y = SMP_FDIV(SMP_FADD(m12, m21), S);
        q.z = SMP_FMUL(0.25f, S);
    }
    return q;
}

SMP_HD float qdot(const Quat &a, const Quat &b)
{
    return SMP_FADD(SMP_FADD(SMP_FMUL(a.w, b.w), SMP_FMUL(a.x, b.x)), SMP_FADD(SMP_FMUL(a.y, b.y), SMP_FMUL(a.z, b.z)));
}

SMP_HD Quat qscale(const Quat &a, float s) { return {SMP_FMUL(a.w, s), SMP_FMUL(a.x, s), SMP_FMUL(a.y, s), SMP_FMUL(a.z, s)}; }
SMP_HD Quat qadd(const Quat &a, const Quat &b) { return {SMP_FADD(a.w, b.w), SMP_FADD(a.x, b.x), SMP_FADD(a.y, b.y), SMP_FADD(a.z, b.z)}; }

SMP_HD Quat qnormalize(const Quat &a)
{
    const float len = SMP_FSQRT(qdot(a, a));
    if (len <= 0.0f) return {1.0f, 0.0f, 0.0f, 0.0f};
    return {SMP_FDIV(a.w, len), SMP_FDIV(a.x, len), SMP_FDIV(a.y, len), SMP_FDIV(a.z, len)};
}

/* slerp along the shorter arc; linear mix when the two are within
 * FLT_EPSILON of parallel */
SMP_HD Quat qslerp(const Quat &x, const Quat &y, float t)
{
    Quat z = y;
    float ct = qdot(x, y);
    if (ct < 0.0f) {
        z = {-y.w, -y.x, -y.y, -y.z};
        ct = -ct;
    }
    if (ct > SMP_FSUB(1.0f, 1.1920928955078125e-7f))
        return qadd(qscale(x, SMP_FSUB(1.0f, t)), qscale(z, t));
    const float ang = acosf_d(ct);
    const float a = sinf_d(SMP_FMUL(SMP_FSUB(1.0f, t), ang)), b = sinf_d(SMP_FMUL(t, ang)), s = sinf_d(ang);
    const Quat n = qadd(qscale(x, a), qscale(z, b));
    return {SMP_FDIV(n.w, s), SMP_FDIV(n.x, s), SMP_FDIV(n.y, s), SMP_FDIV(n.z, s)};
}

/* camera_slerp: rotation slerped, translation mixed a + (b - a) t
 * (include/util/helper_math_extension.h:188-191); out is a row-major 3x4
 * cam2world */
SMP_HD void camera_slerp(const float *a, const float *b, float t, float *out)
{
    const Quat q = qnormalize(qslerp(qnormalize(quat_from(a)), qnormalize(quat_from(b)), t));
    const float qxx = SMP_FMUL(q.x, q.x), qyy = SMP_FMUL(q.y, q.y), qzz = SMP_FMUL(q.z, q.z);
    const float qxz = SMP_FMUL(q.x, q.z), qxy = SMP_FMUL(q.x, q.y), qyz = SMP_FMUL(q.y, q.z);
    const float qwx = SMP_FMUL(q.w, q.x), qwy = SMP_FMUL(q.w, q.y), qwz = SMP_FMUL(q.w, q.z);
    out[0] = SMP_FSUB(1.0f, SMP_FMUL(2.0f, SMP_FADD(qyy, qzz)));
    out[1] = SMP_FMUL(2.0f, SMP_FSUB(qxy, qwz));
    out[2] = SMP_FMUL(2.0f, SMP_FADD(qxz, qwy));
    out[4] = SMP_FMUL(2.0f, SMP_FADD(qxy, qwz));
    out[5] = SMP_FSUB(1.0f, SMP_FMUL(2.0f, SMP_FADD(qxx, qzz)));
    out[6] = SMP_FMUL(2.0f, SMP_FSUB(qyz, qwx));
    out[8] = SMP_FMUL(2.0f, SMP_FSUB(qxz, qwy));
    out[9] = SMP_FMUL(2.0f, SMP_FADD(qyz, qwx));
    out[10] = SMP_FSUB(1.0f, SMP_FMUL(2.0f, SMP_FADD(qxx, qyy)));
    for (int r = 0; r < 3; ++r) out[4 * r + 3] = SMP_FADD(a[4 * r + 3], SMP_FMUL(SMP_FSUB(b[4 * r + 3], a[4 * r + 3]), t));
}

}  // namespace fvc_smp
