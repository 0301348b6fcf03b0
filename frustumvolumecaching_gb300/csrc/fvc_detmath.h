/*
 * fvc_detmath.h - float arithmetic with a fixed operation sequence on the host
 * and on the device.
 *
 * The marcher's index math (step grid, occupancy lookups, froxel coordinates)
 * must give identical bits on the CPU oracle and on the GPU.  Every operation
 * here is a single IEEE-754 binary32 operation with round-to-nearest-even
 * (add, sub, mul, div, sqrt, fma), spelled as an intrinsic on the device so the
 * compiler cannot contract or reorder it; host code including this header is
 * compiled with -ffp-contract=off.
 *
 * log and exp are written here from their mathematical definitions because
 * libm (host) and the CUDA math library (device) round differently:
 *   log x = e*ln2 + 2*atanh(s),  s = (m-1)/(m+1),  x = m*2^e, m in [1/sqrt2, sqrt2),
 *           atanh s = s + s^3/3 + s^5/5 + ... (Taylor series, truncated after s^11);
 *   exp x = 2^k * exp(r),  k = rint(x/ln2),  r = x - k*ln2 (Cody-Waite two-part ln2),
 *           exp r = sum r^n/n!, n <= 8.
 * Both stay within a few ulp of the exact values over the marcher's range.
 */
#ifndef FVC_DETMATH_H
#define FVC_DETMATH_H

#include <math.h>

#if defined(__CUDACC__)
#define FVC_HD __host__ __device__ __forceinline__
#else
#define FVC_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define F_ADD(a, b) __fadd_rn((a), (b))
#define F_SUB(a, b) __fsub_rn((a), (b))
#define F_MUL(a, b) __fmul_rn((a), (b))
#define F_DIV(a, b) __fdiv_rn((a), (b))
#define F_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define F_SQRT(a) __fsqrt_rn((a))
#else
FVC_HD float fvc_h_add(float a, float b) { return a + b; }
FVC_HD float fvc_h_sub(float a, float b) { return a - b; }
FVC_HD float fvc_h_mul(float a, float b) { return a * b; }
FVC_HD float fvc_h_div(float a, float b) { return a / b; }
#define F_ADD(a, b) fvc_h_add((a), (b))
#define F_SUB(a, b) fvc_h_sub((a), (b))
#define F_MUL(a, b) fvc_h_mul((a), (b))
#define F_DIV(a, b) fvc_h_div((a), (b))
#define F_FMA(a, b, c) fmaf((a), (b), (c))
#define F_SQRT(a) sqrtf((a))
#endif

/* ln 2 split so that k*LN2_HI is exact for |k| < 2^11 (LN2_HI has 16
 * significant bits); LN2_LO = ln 2 - LN2_HI rounded to binary32. */
#define FVC_LN2_HI 0.693145751953125f
#define FVC_LN2_LO 1.42860682030941723212e-06f
#define FVC_INV_LN2 1.44269504088896340736f

/* Natural log of a positive finite x; +inf -> +inf, 0 -> -inf, x<0 -> NaN. */
FVC_HD float fvc_logf(float x)
{
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int e;
    float m = frexpf(x, &e); /* x = m * 2^e, m in [0.5, 1), exact */
    if (m < 0.70710678118654752f) { m = F_MUL(m, 2.0f); e -= 1; }
    const float s = F_DIV(F_SUB(m, 1.0f), F_ADD(m, 1.0f));
    const float s2 = F_MUL(s, s);
    /* q = 1/3 + s2/5 + s2^2/7 + s2^3/9 + s2^4/11 (Horner) */
    float q = 1.0f / 11.0f;
    q = F_FMA(q, s2, 1.0f / 9.0f);
    q = F_FMA(q, s2, 1.0f / 7.0f);
    q = F_FMA(q, s2, 1.0f / 5.0f);
    q = F_FMA(q, s2, 1.0f / 3.0f);
    const float two_s = F_MUL(2.0f, s);
    const float log_m = F_FMA(F_MUL(two_s, s2), q, two_s);
    const float ef = (float)e;
    return F_ADD(F_MUL(ef, FVC_LN2_HI), F_FMA(ef, FVC_LN2_LO, log_m));
}

/* e^x for finite x; underflows to 0 below -103.9, overflows to +inf above 88.73. */
FVC_HD float fvc_expf(float x)
{
    if (x != x) return x;
    if (x > 88.7228f) return INFINITY;
    if (x < -103.9721f) return 0.0f;
    const float kf = rintf(F_MUL(x, FVC_INV_LN2));
    float r = F_FMA(-kf, FVC_LN2_HI, x);
    r = F_FMA(-kf, FVC_LN2_LO, r);
    float p = 1.0f / 40320.0f;
    p = F_FMA(p, r, 1.0f / 5040.0f);
    p = F_FMA(p, r, 1.0f / 720.0f);
    p = F_FMA(p, r, 1.0f / 120.0f);
    p = F_FMA(p, r, 1.0f / 24.0f);
    p = F_FMA(p, r, 1.0f / 6.0f);
    p = F_FMA(p, r, 0.5f);
    p = F_FMA(p, r, 1.0f);
    p = F_FMA(p, r, 1.0f);
    return ldexpf(p, (int)kf);
}

/* (1+c)^e given L = log(1+c) as L_hi + L_lo (L_hi = (float)L,
 * L_lo = (float)(L - L_hi) from a double log): exp(e*L) with the rounding
 * error of e*L_hi recovered by an fma and applied to first order. */
FVC_HD float fvc_pow_1pc(float e, float L_hi, float L_lo)
{
    const float p = F_MUL(e, L_hi);
    const float perr = F_FMA(e, L_lo, F_FMA(e, L_hi, -p));
    const float r = fvc_expf(p);
    return F_FMA(r, perr, r);
}

#endif /* FVC_DETMATH_H */
