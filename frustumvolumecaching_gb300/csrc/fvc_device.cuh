/*
 * fvc_device.cuh - device-side marcher math, hash-grid encoding and the
 * warp-level fused MLP of the GB300 renderer.
 *
 * Marcher index math uses the F_* single-rounding intrinsics of
 * fvc_detmath.h in the reference's operation order
 * (include/raymarch_common.h, include/common.h) so per-ray step sequences,
 * occupancy lookups and froxel coordinates are bit-identical to the CPU
 * oracle.  The network runs on the tensor cores (mma.sync m16n8k16, fp16
 * inputs, fp32 accumulation); layer outputs are rounded to fp16 between
 * layers as the reference's fp16 network stores them.
 */
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "fvc_detmath.h"
#include "fvc_sampling.h"

namespace fvc {

/* --------------------------------------------------------------------- */
/* parameter blocks (filled on the host from the C-ABI structs)           */
/* --------------------------------------------------------------------- */
struct DevScene {
    float3 aabb_from, aabb_to;
    float3 unit_off;  /* aabb_from / 2^(nlvl-1)             (world_to_aabb_unit) */
    float3 unit_den;  /* (aabb_to - aabb_from) / 2^(nlvl-1) */
    float3 aabb_den;  /* aabb_to - aabb_from                 (contract_aabb)      */
    float3 c_from, c_den; /* contraction aabb and its extent */
    float3 unit_rcp, aabb_rcp, c_rcp; /* correctly rounded 1 / unit_den, 1 / aabb_den, 1 / c_den (div_rn_by) */
    int nlvl, normalized, contraction, is_open_gl;
    float alpha_thre;
};

struct DevSteps {
    float cone, log1p_c, log1p_c_lo, near_, near_i, far_;
    float dt_min, dt_max, t_min, t_max, i_min, i_max;
};

struct DevCam {
    int W, H, gl;
    float fx, fy, px, py;
    float c2w[12];
    float w2c[12];
    /* RaymarchInfo's sampling: nd = 1 when not deterministic (pixel and start
     * jitter, depth of field when aperature != 0), motion_blur toward nc2w */
    int nd, motion_blur, sample_index;
    float aperature, focus_z;
    float nc2w[12];
};

constexpr int MAX_LEVELS = 16;
struct DevGrid {
    int n_levels;
    int F;                /* features per level: 2 (16 levels) or 4 (8 levels); offset[] counts half2 */
    uint32_t dense_mask;
    float scale[MAX_LEVELS];
    uint32_t res[MAX_LEVELS], res2[MAX_LEVELS], size[MAX_LEVELS], offset[MAX_LEVELS];
};

/* fragment-ordered weights (uint2 per lane per (n-tile, k-step)) */
constexpr int W_L1 = 0;                  /* 64 x 32  : 8 ntiles * 2 ksteps * 32 lanes */
constexpr int W_L2 = W_L1 + 8 * 2 * 32;  /* 16 x 64  : 2 * 4 * 32 */
constexpr int W_L3 = W_L2 + 2 * 4 * 32;  /* 64 x 32  (head input: base16 | sh16) */
constexpr int W_L4 = W_L3 + 8 * 2 * 32;  /* 64 x 64 */
constexpr int W_L5 = W_L4 + 8 * 4 * 32;  /* 16 x 64 */
constexpr int W_TOTAL = W_L5 + 2 * 4 * 32; /* uint2 entries = 2560 -> 20 KiB */

/* --------------------------------------------------------------------- */
/* step grid (StepsizeInfo, include/common.h:133-163)                     */
/* --------------------------------------------------------------------- */
__device__ __forceinline__ float t_from_step(const DevSteps &s, float step)
{
    if (s.cone <= 0.0f) return F_MUL(step, s.dt_min);
    if (step >= s.i_max) return F_ADD(s.t_max, F_MUL(F_SUB(step, s.i_max), s.dt_max));
    if (step < s.i_min) return F_MUL(step, s.dt_min);
    return F_MUL(s.t_min, fvc_pow_1pc(F_SUB(step, s.i_min), s.log1p_c, s.log1p_c_lo));
}

__device__ __forceinline__ float step_from_t(const DevSteps &s, float t)
{
    if (s.cone <= 0.0f) return F_DIV(t, s.dt_min);
    if (t >= s.t_max) return F_ADD(F_DIV(F_SUB(t, s.t_max), s.dt_max), s.i_max);
    if (t < s.t_min) return F_DIV(t, s.dt_min);
    return F_ADD(F_DIV(fvc_logf(F_DIV(t, s.t_min)), s.log1p_c), s.i_min);
}

/* calculate_stepsize, include/raymarch_common.h:274-284 */
__device__ __forceinline__ float calc_step(const DevSteps &s, float t)
{
    return fmaxf(s.dt_min, fminf(F_MUL(t, s.cone), s.dt_max));
}

/* valid_t_from_t, include/raymarch_common.h:286-296 */
__device__ __forceinline__ float valid_t_from_t(const DevSteps &s, float t)
{
    return t_from_step(s, F_ADD(roundf(F_SUB(step_from_t(s, fmaxf(t, s.near_)), s.near_i)), s.near_i));
}

/* --------------------------------------------------------------------- */
/* rays                                                                   */
/* --------------------------------------------------------------------- */
__device__ __forceinline__ float dot4(float ax, float ay, float az, float aw, const float *m)
{
    return F_ADD(F_ADD(F_ADD(F_MUL(ax, m[0]), F_MUL(ay, m[1])), F_MUL(az, m[2])), F_MUL(aw, m[3]));
}
__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    return F_ADD(F_ADD(F_MUL(a.x, b.x), F_MUL(a.y, b.y)), F_MUL(a.z, b.z));
}
__device__ __forceinline__ float3 at(float3 o, float3 d, float t)
{
    return make_float3(F_ADD(o.x, F_MUL(t, d.x)), F_ADD(o.y, F_MUL(t, d.y)), F_ADD(o.z, F_MUL(t, d.z)));
}

/* x / d rounded to nearest, from r = RN(1 / d): q0 = RN(x r), the exact
 * residual e = x - q0 d by one fused multiply-add, q = RN(q0 + e r).  With a
 * correctly rounded reciprocal this is the correctly rounded quotient
 * (Markstein, "Computation of elementary functions on the IBM RISC
 * System/6000 processor", IBM J. Res. Dev. 1990) for operands away from
 * overflow and underflow: the same bits as the IEEE division, in three
 * instructions when d is fixed and r computed once.  The scene's
 * denominators come with their reciprocals; a per-ray denominator takes one
 * __frcp_rn. */
__device__ __forceinline__ float div_rn_by(float x, float d, float r)
{
    const float q0 = __fmul_rn(x, r);
    const float e = __fmaf_rn(-q0, d, x);
    return __fmaf_rn(e, r, q0);
}

/* generateRay for the pixel centre (deterministic), include/raymarch_common.h:190-251;
 * normalize() uses the correctly rounded 1/sqrt (double, rounded once). */
__device__ __forceinline__ void generate_ray(const DevCam &c, int x, int y, float3 &o, float3 &d)
{
    const float sx = F_ADD((float)x, 0.5f), sy = F_ADD((float)y, 0.5f);
    const float sgn = c.gl ? -1.f : 1.f;
    const float dx = F_DIV(F_SUB(sx, c.px), c.fx);
    const float dy = F_MUL(F_DIV(F_SUB(sy, c.py), c.fy), sgn);
    const float dz = sgn;
    float3 v = make_float3(dot4(dx, dy, dz, 0.f, c.c2w), dot4(dx, dy, dz, 0.f, c.c2w + 4), dot4(dx, dy, dz, 0.f, c.c2w + 8));
    const float inv = __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn((double)dot3(v, v))));
    d = make_float3(F_MUL(v.x, inv), F_MUL(v.y, inv), F_MUL(v.z, inv));
    o = make_float3(c.c2w[3], c.c2w[7], c.c2w[11]);
}

/* generateRay with RaymarchInfo's sampling (include/raymarch_common.h:218-251,
 * src/renderer.cu:105-108): the deterministic pixel centre, or the pixel plus
 * ld_random_pixel_offset, the camera slerped toward next_cam_info for motion
 * blur (ld_random_val seeded by the pixel index) and the thin-lens offset of
 * depth of field (the direction then (lookat - origin) / focus_z, not
 * renormalised, as the reference leaves it).  fvc_sampling.h holds the
 * sampling arithmetic, shared with the oracle. */
__device__ __forceinline__ void generate_ray_rm(const DevCam &c, int x, int y, float3 &o, float3 &d)
{
    if (!c.nd) {
        generate_ray(c, x, y, o, d);
        return;
    }
    float ox, oy;
    fvc_smp::pixel_offset((uint32_t)c.sample_index, ox, oy);
    const float sx = F_ADD((float)x, ox), sy = F_ADD((float)y, oy);
    float m[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) m[k] = c.c2w[k];
    if (c.motion_blur) {
        const float tm = fvc_smp::ld_val((uint32_t)c.sample_index, (uint32_t)(y * c.W + x) * 72239731u);
        fvc_smp::camera_slerp(c.c2w, c.nc2w, tm, m);
    }
    const float sgn = c.gl ? -1.f : 1.f;
    const float dx = F_DIV(F_SUB(sx, c.px), c.fx);
    const float dy = F_MUL(F_DIV(F_SUB(sy, c.py), c.fy), sgn);
    const float dz = sgn;
    float3 v = make_float3(dot4(dx, dy, dz, 0.f, m), dot4(dx, dy, dz, 0.f, m + 4), dot4(dx, dy, dz, 0.f, m + 8));
    const float inv = __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn((double)dot3(v, v))));
    d = make_float3(F_MUL(v.x, inv), F_MUL(v.y, inv), F_MUL(v.z, inv));
    o = make_float3(m[3], m[7], m[11]);
    if (c.aperature != 0.0f) {
        const float3 look = make_float3(F_ADD(o.x, F_MUL(d.x, c.focus_z)), F_ADD(o.y, F_MUL(d.y, c.focus_z)),
                                        F_ADD(o.z, F_MUL(d.z, c.focus_z)));
        float bx, by;
        fvc_smp::lens_offset((uint32_t)c.sample_index, sx, sy, c.W, c.H, c.aperature, bx, by);
        o.x = F_ADD(o.x, F_ADD(F_MUL(m[0], bx), F_MUL(m[1], by)));
        o.y = F_ADD(o.y, F_ADD(F_MUL(m[4], bx), F_MUL(m[5], by)));
        o.z = F_ADD(o.z, F_ADD(F_MUL(m[8], bx), F_MUL(m[9], by)));
        d = make_float3(F_DIV(F_SUB(look.x, o.x), c.focus_z), F_DIV(F_SUB(look.y, o.y), c.focus_z),
                        F_DIV(F_SUB(look.z, o.z), c.focus_z));
    }
}

/* ray_aabb_intersect, include/raymarch_common.h:482-532 */
__device__ __forceinline__ bool ray_aabb(float3 o, float3 d, float3 from, float3 to, float &tn, float &tf)
{
    float tmin = F_DIV(F_SUB(from.x, o.x), d.x), tmax = F_DIV(F_SUB(to.x, o.x), d.x);
    if (tmin > tmax) { float c = tmin; tmin = tmax; tmax = c; }
    float tymin = F_DIV(F_SUB(from.y, o.y), d.y), tymax = F_DIV(F_SUB(to.y, o.y), d.y);
    if (tymin > tymax) { float c = tymin; tymin = tymax; tymax = c; }
    if (tmin > tymax || tymin > tmax) { tn = 1e10f; tf = 1e10f; return false; }
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = F_DIV(F_SUB(from.z, o.z), d.z), tzmax = F_DIV(F_SUB(to.z, o.z), d.z);
    if (tzmin > tzmax) { float c = tzmin; tzmin = tzmax; tzmax = c; }
    if (tmin > tzmax || tzmin > tmax) { tn = 1e10f; tf = 1e10f; return false; }
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    tn = tmin; tf = tmax;
    return true;
}

/* transformRay, include/raymarch_common.h:253-262 */
__device__ __forceinline__ void transform_ray(const float *m, float3 o, float3 d, float3 &oc, float3 &dc)
{
    oc = make_float3(dot4(o.x, o.y, o.z, 1.0f, m), dot4(o.x, o.y, o.z, 1.0f, m + 4), dot4(o.x, o.y, o.z, 1.0f, m + 8));
    dc = make_float3(dot4(d.x, d.y, d.z, 0.0f, m), dot4(d.x, d.y, d.z, 0.0f, m + 4), dot4(d.x, d.y, d.z, 0.0f, m + 8));
}

/* --------------------------------------------------------------------- */
/* occupancy grid (grid_occupied_at<128, true>, include/raymarch_common.h:660-710) */
/* --------------------------------------------------------------------- */
/* morton3D's bit spreading (include/raymarch_common.h:98-110) for the cell
 * indices this grid produces, 0..128: for inputs below 256 the 10-bit
 * spreading's first step (v * 0x00010001 & 0xFF0000FF) is the identity, so
 * the three remaining steps give the same bits. */
__device__ __forceinline__ uint32_t expand_bits3(uint32_t v)
{
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

/* mip_from_unit's cascade of a point whose largest offset from the grid
 * centre is mx (finite, >= 0): max(0, frexp exponent of mx + 1), read from
 * the exponent field.  A zero or subnormal mx reads -126 (its frexp exponent
 * is at most -126) and gives mip 0 like frexpf. */
__device__ __forceinline__ int mip_of(float mx)
{
    return max(0, (int)(__float_as_uint(mx) >> 23) - 125);
}

/* Cell index along one axis at cascade mip, for a = unit coordinate - 1/2
 * with |a| < 2^(mip-1): (int)((a * 2^-mip + 1/2) * 128) as the reference
 * evaluates it, rounded once.  a * 2^-mip and the final * 128 are exact
 * (powers of two), and rounding commutes with a power-of-two scale away from
 * overflow and underflow, so RN(a 2^-mip + 1/2) * 128 = RN(a 2^(7-mip) + 64),
 * one fused multiply-add with the same bits.  The result lies in [0, 128]. */
__device__ __forceinline__ int cell_of(float a, int mip)
{
    return (int)__fmaf_rn(a, __int_as_float((134 - mip) << 23), 64.0f);
}

__device__ __forceinline__ bool occupied(const DevScene &sc, const uint8_t *__restrict__ bits, float3 p)
{
    float3 u = p;
    if (!sc.normalized)
        u = make_float3(div_rn_by(F_SUB(p.x, sc.unit_off.x), sc.unit_den.x, sc.unit_rcp.x),
                        div_rn_by(F_SUB(p.y, sc.unit_off.y), sc.unit_den.y, sc.unit_rcp.y),
                        div_rn_by(F_SUB(p.z, sc.unit_off.z), sc.unit_den.z, sc.unit_rcp.z));
    const float ax = F_SUB(u.x, 0.5f), ay = F_SUB(u.y, 0.5f), az = F_SUB(u.z, 0.5f);
    const float mx = fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fabsf(az));
    if (!(mx <= 3.0e38f)) return false; /* NaN / inf positions never index the grid */
    const int mip = mip_of(mx);
    if (mip >= sc.nlvl) return false;
    const int ix = cell_of(ax, mip), iy = cell_of(ay, mip), iz = cell_of(az, mip);
    const uint32_t idx = expand_bits3((uint32_t)ix) | (expand_bits3((uint32_t)iy) << 1) | (expand_bits3((uint32_t)iz) << 2);
    const uint32_t bidx = idx / 8u + (uint32_t)((128 * 128 * 128 / 8) * mip);
    return (__ldg(bits + bidx) >> (idx & 7u)) & 1u;
}

/* occupied() plus, for an empty cell, the extent of empty space along the
 * ray: the DDA of grid_occupied_at's t_dist_to_next_voxel form
 * (include/raymarch_common.h:712-744), made conservative so that skipping
 * never changes a result.  t_free receives a t below which every point
 * o + t d (t >= the query's) lies in the same empty cell by the same
 * arithmetic occupied() uses: the cell's exit face along each axis less a
 * margin of 1/1024 of the cell (in world units, far above the float rounding
 * of the point, of its unit coordinates and of the cell index), and no skip
 * at all (t_free = -inf) when the point itself is within that margin of a
 * face or the cell is outside the grid.  A cell narrower than 4 steps (dt,
 * the query's step) is not skipped: computing its bound costs about what
 * the lookups it saves do.  Cells of one mip level never
 * straddle a cascade boundary (the inner cascade covers cells 32..95 of the
 * outer one), so a mip-m cell's points all index mip m. */
__device__ __forceinline__ bool occupied_skip(const DevScene &sc, const uint8_t *__restrict__ bits, float3 o, float3 d,
                                              float3 inv_d, float t, float dt, float &t_free)
{
    const float3 p = at(o, d, t);
    float3 u = p;
    if (!sc.normalized)
        u = make_float3(div_rn_by(F_SUB(p.x, sc.unit_off.x), sc.unit_den.x, sc.unit_rcp.x),
                        div_rn_by(F_SUB(p.y, sc.unit_off.y), sc.unit_den.y, sc.unit_rcp.y),
                        div_rn_by(F_SUB(p.z, sc.unit_off.z), sc.unit_den.z, sc.unit_rcp.z));
    const float ax = F_SUB(u.x, 0.5f), ay = F_SUB(u.y, 0.5f), az = F_SUB(u.z, 0.5f);
    const float mx = fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fabsf(az));
    t_free = -1e30f;
    if (!(mx <= 3.0e38f)) return false;
    const int mip = mip_of(mx);
    if (mip >= sc.nlvl) return false;
    const int ix = cell_of(ax, mip), iy = cell_of(ay, mip), iz = cell_of(az, mip);
    const uint32_t idx = expand_bits3((uint32_t)ix) | (expand_bits3((uint32_t)iy) << 1) | (expand_bits3((uint32_t)iz) << 2);
    const uint32_t bidx = idx / 8u + (uint32_t)((128 * 128 * 128 / 8) * mip);
    if ((__ldg(bits + bidx) >> (idx & 7u)) & 1u) return true;
    /* the empty cell's faces in world units: unit a = (i / 128 - 1/2) 2^mip + 1/2 */
    const float cell = __int_as_float((127 + mip - 7) << 23); /* 2^mip / 128, in unit coordinates */
    const float den[3] = {sc.normalized ? 1.f : sc.unit_den.x, sc.normalized ? 1.f : sc.unit_den.y, sc.normalized ? 1.f : sc.unit_den.z};
    /* cells that span fewer than 4 steps along the ray are cheaper to look up step by step */
    if (cell * fminf(fminf(den[0], den[1]), den[2]) < 4.0f * dt * fmaxf(fmaxf(fabsf(d.x), fabsf(d.y)), fabsf(d.z))) return false;
    const float off[3] = {sc.normalized ? 0.f : sc.unit_off.x, sc.normalized ? 0.f : sc.unit_off.y, sc.normalized ? 0.f : sc.unit_off.z};
    const int ic[3] = {ix, iy, iz};
    const float pc[3] = {p.x, p.y, p.z}, oc[3] = {o.x, o.y, o.z}, dc[3] = {d.x, d.y, d.z}, ic_inv[3] = {inv_d.x, inv_d.y, inv_d.z};
    const float half = __int_as_float((127 + mip - 1) << 23); /* 2^mip / 2 */
    float tf = 1e30f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float lo_u = (float)ic[k] * cell - half + 0.5f, hi_u = lo_u + cell;
        const float lo = off[k] + lo_u * den[k], hi = off[k] + hi_u * den[k];
        const float margin = cell * den[k] * (1.0f / 1024.0f);
        if (!(pc[k] - lo > margin && hi - pc[k] > margin)) return false; /* too close to a face: no skip */
        if (dc[k] > 0.f) tf = fminf(tf, (hi - margin - oc[k]) * ic_inv[k]);
        else if (dc[k] < 0.f) tf = fminf(tf, (lo + margin - oc[k]) * ic_inv[k]);
    }
    t_free = tf;
    return false;
}

/* apply_contraction, include/raymarch_common.h:610-653 */
__device__ __forceinline__ float3 contract(const DevScene &sc, float3 p)
{
    if (sc.contraction == 1)
        return make_float3(div_rn_by(F_SUB(p.x, sc.aabb_from.x), sc.aabb_den.x, sc.aabb_rcp.x),
                           div_rn_by(F_SUB(p.y, sc.aabb_from.y), sc.aabb_den.y, sc.aabb_rcp.y),
                           div_rn_by(F_SUB(p.z, sc.aabb_from.z), sc.aabb_den.z, sc.aabb_rcp.z));
    if (sc.contraction == 2 || sc.contraction == 3) {
        const float ux = F_SUB(F_MUL(div_rn_by(F_SUB(p.x, sc.c_from.x), sc.c_den.x, sc.c_rcp.x), 2.0f), 1.0f);
        const float uy = F_SUB(F_MUL(div_rn_by(F_SUB(p.y, sc.c_from.y), sc.c_den.y, sc.c_rcp.y), 2.0f), 1.0f);
        const float uz = F_SUB(F_MUL(div_rn_by(F_SUB(p.z, sc.c_from.z), sc.c_den.z, sc.c_rcp.z), 2.0f), 1.0f);
        const float n = sc.contraction == 3 ? fmaxf(fmaxf(fabsf(ux), fabsf(uy)), fabsf(uz))
                                            : F_SQRT(F_ADD(F_ADD(F_MUL(ux, ux), F_MUL(uy, uy)), F_MUL(uz, uz)));
        const float f = fmaxf(n, 1.0f);
        /* 1 / f is the correctly rounded reciprocal (the IEEE 1.0f / f); / 4 is an exact * 0.25 */
        const float rf = __frcp_rn(f);
        const float k = F_SUB(2.0f, rf);
        return make_float3(F_ADD(F_MUL(F_MUL(k, div_rn_by(ux, f, rf)), 0.25f), 0.5f),
                           F_ADD(F_MUL(F_MUL(k, div_rn_by(uy, f, rf)), 0.25f), 0.5f),
                           F_ADD(F_MUL(F_MUL(k, div_rn_by(uz, f, rf)), 0.25f), 0.5f));
    }
    return p;
}

/* cam2froxel, include/raymarch_common.h:316-329, in two parts: the image
 * coordinates and the distance t, and the depth coordinate (the step index
 * of t, the costly part), which a caller can leave until it needs it */
__device__ __forceinline__ float2 cam2froxel_xy(float3 c, const DevCam &cam, float &t)
{
    const float sgn = cam.gl ? -1.f : 1.f;
    const float z = F_MUL(c.z, sgn), rz = __frcp_rn(z);
    t = F_SQRT(dot3(c, c));
    return make_float2(F_ADD(F_MUL(div_rn_by(c.x, z, rz), cam.fx), cam.px), F_ADD(F_MUL(div_rn_by(F_MUL(c.y, sgn), z, rz), cam.fy), cam.py));
}
__device__ __forceinline__ float froxel_z(const DevSteps &st, float t, float cz)
{
    return F_MUL(F_SUB(step_from_t(st, t), st.near_i), cz < 0.0f ? -1.0f : 1.0f);
}
__device__ __forceinline__ float3 cam2froxel(float3 c, const DevCam &cam, const DevSteps &st, float &t)
{
    const float2 xy = cam2froxel_xy(c, cam, t);
    return make_float3(xy.x, xy.y, froxel_z(st, t, c.z));
}

/* --------------------------------------------------------------------- */
/* hash grid (Instant-NGP multiresolution hash encoding)                  */
/* --------------------------------------------------------------------- */
/* packed fp32 pair arithmetic of sm_100+ (add/sub/fma .f32x2 on a 64-bit register pair) */
__device__ __forceinline__ unsigned long long f2_bits(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 f2_from_bits(unsigned long long r)
{
    float2 a;
    asm("mov.b64 {%0,%1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
/* a + t * (b - a), each step rounded to nearest */
__device__ __forceinline__ float2 f2_lerp(float2 a, float2 b, float t)
{
    unsigned long long d, r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(b)), "l"(f2_bits(a)));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_bits(make_float2(t, t))), "l"(d), "l"(f2_bits(a)));
    return f2_from_bits(r);
}

/* Encodes one position into 2*n_levels features (fp16) written to
 * out[0 .. 2*n_levels) as half2 per level.  Corner and fraction in float32
 * (p = fma(scale, x, 0.5), floor, subtract); the trilinear interpolation in
 * float32 as lerps along x, y, z (the same weighted sum of the 8 corners).
 * Levels are processed in groups of LG: the 8*LG corner loads of a group are
 * all issued before any of them is consumed, so a thread keeps 8*LG gathers
 * in flight instead of 8. */
/* the 4-feature grid (instant-ngp's 8 levels x 4 features): an entry is two
 * half2 (one 8-byte gather per corner), the level's features go to
 * out[2l], out[2l + 1]; levels in groups of LG / 2 */
template <int LG>
__device__ __forceinline__ void hash_encode_levels_f4(const DevGrid &g, const __half2 *__restrict__ table, float3 pos, __half2 *out,
                                                      int l_begin, int l_end)
{
    constexpr int G = LG / 2 > 0 ? LG / 2 : 1;
    for (int l0 = l_begin; l0 < l_end; l0 += G) {
        uint2 v[G][8];
        float wx[G], wy[G], wz[G];
#pragma unroll
        for (int j = 0; j < G; ++j) {
            const int l = l0 + j;
            const float sc = g.scale[l];
            const float px = __fmaf_rn(sc, pos.x, 0.5f), py = __fmaf_rn(sc, pos.y, 0.5f), pz = __fmaf_rn(sc, pos.z, 0.5f);
            const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
            const uint32_t gx = (uint32_t)(int)fx, gy = (uint32_t)(int)fy, gz = (uint32_t)(int)fz;
            wx[j] = __fsub_rn(px, fx); wy[j] = __fsub_rn(py, fy); wz[j] = __fsub_rn(pz, fz);
            const uint32_t size = g.size[l];
            const uint2 *tl = reinterpret_cast<const uint2 *>(table + g.offset[l]);
            if ((g.dense_mask >> l) & 1u) {
                const uint32_t r = g.res[l], r2 = g.res2[l];
                const uint32_t b = gx + gy * r + gz * r2;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    uint32_t i = b + ((c & 1) ? 1u : 0u) + ((c & 2) ? r : 0u) + ((c & 4) ? r2 : 0u);
                    if (i >= size) i -= size;
                    v[j][c] = __ldg(tl + i);
                }
            } else {
                const uint32_t hy0 = gy * 2654435761u, hy1 = (gy + 1u) * 2654435761u;
                const uint32_t hz0 = gz * 805459861u, hz1 = (gz + 1u) * 805459861u;
                const uint32_t m = size - 1u;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    v[j][c] = __ldg(tl + (((gx + ((c & 1) ? 1u : 0u)) ^ ((c & 2) ? hy1 : hy0) ^ ((c & 4) ? hz1 : hz0)) & m));
            }
        }
#pragma unroll
        for (int j = 0; j < G; ++j) {
#pragma unroll
            for (int h = 0; h < 2; ++h) { /* features 0-1, then 2-3 */
                float2 e[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t a = h ? v[j][2 * k].y : v[j][2 * k].x, b = h ? v[j][2 * k + 1].y : v[j][2 * k + 1].x;
                    e[k] = f2_lerp(__half22float2(*reinterpret_cast<const __half2 *>(&a)),
                                   __half22float2(*reinterpret_cast<const __half2 *>(&b)), wx[j]);
                }
                const float2 g0 = f2_lerp(e[0], e[1], wy[j]), g1 = f2_lerp(e[2], e[3], wy[j]);
                out[2 * (l0 + j) + h] = __float22half2_rn(f2_lerp(g0, g1, wz[j]));
            }
        }
    }
}

template <int LG = 4>
__device__ __forceinline__ void hash_encode_levels(const DevGrid &g, const __half2 *__restrict__ table, float3 pos, __half2 *out,
                                                   int l_begin, int l_end)
{
    if (g.F == 4) {
        hash_encode_levels_f4<LG>(g, table, pos, out, l_begin, l_end);
        return;
    }
    for (int l0 = l_begin; l0 < l_end; l0 += LG) {
        __half2 v[LG][8];
        float wx[LG], wy[LG], wz[LG];
#pragma unroll
        for (int j = 0; j < LG; ++j) {
            const int l = l0 + j;
            const float sc = g.scale[l];
            const float px = __fmaf_rn(sc, pos.x, 0.5f), py = __fmaf_rn(sc, pos.y, 0.5f), pz = __fmaf_rn(sc, pos.z, 0.5f);
            const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
            const uint32_t gx = (uint32_t)(int)fx, gy = (uint32_t)(int)fy, gz = (uint32_t)(int)fz;
            wx[j] = __fsub_rn(px, fx); wy[j] = __fsub_rn(py, fy); wz[j] = __fsub_rn(pz, fz);
            const uint32_t size = g.size[l];
            const __half2 *tl = table + g.offset[l];
            if ((g.dense_mask >> l) & 1u) {
                const uint32_t r = g.res[l], r2 = g.res2[l];
                const uint32_t b = gx + gy * r + gz * r2;
                if (b + 1u + r + r2 < size) { /* no corner reaches past the table (all but the grid's far faces) */
#pragma unroll
                    for (int c = 0; c < 8; ++c) v[j][c] = __ldg(tl + (b + ((c & 1) ? 1u : 0u) + ((c & 2) ? r : 0u) + ((c & 4) ? r2 : 0u)));
                } else {
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        uint32_t i = b + ((c & 1) ? 1u : 0u) + ((c & 2) ? r : 0u) + ((c & 4) ? r2 : 0u);
                        if (i >= size) i -= size; /* == i % size: dense indices stay below 2*size */
                        v[j][c] = __ldg(tl + i);
                    }
                }
            } else {
                const uint32_t hy0 = gy * 2654435761u, hy1 = (gy + 1u) * 2654435761u;
                const uint32_t hz0 = gz * 805459861u, hz1 = (gz + 1u) * 805459861u;
                const uint32_t m = size - 1u; /* hashed levels hold 2^log2_T entries */
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    v[j][c] = __ldg(tl + (((gx + ((c & 1) ? 1u : 0u)) ^ ((c & 2) ? hy1 : hy0) ^ ((c & 4) ? hz1 : hz0)) & m));
            }
        }
#pragma unroll
        for (int j = 0; j < LG; ++j) {
            /* trilinear interpolation as 7 lerps (x, then y, then z) on both features at once */
            float2 e[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) e[k] = f2_lerp(__half22float2(v[j][2 * k]), __half22float2(v[j][2 * k + 1]), wx[j]);
            const float2 g0 = f2_lerp(e[0], e[1], wy[j]), g1 = f2_lerp(e[2], e[3], wy[j]);
            out[l0 + j] = __float22half2_rn(f2_lerp(g0, g1, wz[j]));
        }
    }
}

/* all levels of the grid (features of level l in out[l]) */
template <int LG = 4>
__device__ __forceinline__ void hash_encode(const DevGrid &g, const __half2 *__restrict__ table, float3 pos, __half2 *out)
{
    hash_encode_levels<LG>(g, table, pos, out, 0, g.n_levels);
}

/* SH degree 4 (16 values) of a unit_to_01 direction, written as 8 half2.
 * Real SH of Sloan's "Stupid SH" recurrences, sign convention of
 * src/my_fully_fused_mlp.cu:216-233. */
__device__ __forceinline__ void sh16(float3 d01, __half2 *out)
{
    const float x = d01.x * 2.f - 1.f, y = d01.y * 2.f - 1.f, z = d01.z * 2.f - 1.f;
    const float xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
    out[0] = __floats2half2_rn(0.28209479177387814f, -0.48860251190291987f * y);
    out[1] = __floats2half2_rn(0.48860251190291987f * z, -0.48860251190291987f * x);
    out[2] = __floats2half2_rn(1.0925484305920792f * xy, -1.0925484305920792f * yz);
    out[3] = __floats2half2_rn(0.94617469575755997f * z2 - 0.31539156525251999f, -1.0925484305920792f * xz);
    out[4] = __floats2half2_rn(0.54627421529603959f * x2 - 0.54627421529603959f * y2, 0.59004358992664352f * y * (-3.0f * x2 + y2));
    out[5] = __floats2half2_rn(2.8906114426405538f * xy * z, 0.45704579946446572f * y * (1.0f - 5.0f * z2));
    out[6] = __floats2half2_rn(0.3731763325901154f * z * (5.0f * z2 - 3.0f), 0.45704579946446572f * x * (1.0f - 5.0f * z2));
    out[7] = __floats2half2_rn(1.4453057213202769f * z * (x2 - y2), 0.59004358992664352f * x * (-x2 + 3.0f * y2));
}

/* --------------------------------------------------------------------- */
/* warp MLP on tensor cores                                               */
/* --------------------------------------------------------------------- */
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint2 b)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi)
{
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

/* Tile layout: 32 rows x TILE_STRIDE halfs.
 *   cols  0..31 : hash features (layer-1 input)
 *   cols 16..31 : overwritten with the density-network output (head input part 1)
 *   cols 32..47 : SH of the direction (head input part 2)
 * Stride 56 halfs (112 B) makes the fragment loads bank-conflict free. */
constexpr int TILE_STRIDE = 56;

/* A fragments (m16 x k16) of rows [16*mt, 16*mt+16), cols [c0, c0+16) */
__device__ __forceinline__ void load_a(const __half *tile, int mt, int c0, int lane, uint32_t (&a)[4])
{
    const int g = lane >> 2, t = lane & 3;
    const __half *r0 = tile + (16 * mt + g) * TILE_STRIDE + c0 + 2 * t;
    const __half *r1 = r0 + 8 * TILE_STRIDE;
    a[0] = *reinterpret_cast<const uint32_t *>(r0);
    a[1] = *reinterpret_cast<const uint32_t *>(r1);
    a[2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
    a[3] = *reinterpret_cast<const uint32_t *>(r1 + 8);
}

/* Density network on the 32 rows of a tile: layer 1 (64 x 32, ReLU) and
 * layer 2 (16 x 64).  Writes the fp16 outputs into tile cols 16..31 and
 * returns nothing; col 16 holds the log-density. */
__device__ __forceinline__ void density_mlp(__half *tile, const uint2 *__restrict__ W, int lane)
{
    const int g = lane >> 2, t = lane & 3;
    uint32_t a1[2][2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int s = 0; s < 2; ++s) load_a(tile, mt, 16 * s, lane, a1[mt][s]);
    /* layer 1 -> A fragments of layer 2 (K = 64: 4 k-steps) */
    uint32_t a2[2][4][4];
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
        float c[2][2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) c[mt][h][0] = c[mt][h][1] = c[mt][h][2] = c[mt][h][3] = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const uint2 b = W[W_L1 + ((2 * jp + h) * 2 + s) * 32 + lane];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) mma16816(c[mt][h], a1[mt][s], b);
            }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            a2[mt][jp][0] = pack_h2(fmaxf(c[mt][0][0], 0.f), fmaxf(c[mt][0][1], 0.f));
            a2[mt][jp][1] = pack_h2(fmaxf(c[mt][0][2], 0.f), fmaxf(c[mt][0][3], 0.f));
            a2[mt][jp][2] = pack_h2(fmaxf(c[mt][1][0], 0.f), fmaxf(c[mt][1][1], 0.f));
            a2[mt][jp][3] = pack_h2(fmaxf(c[mt][1][2], 0.f), fmaxf(c[mt][1][3], 0.f));
        }
    }
    __syncwarp();
    /* layer 2: 16 outputs */
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        float c[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) c[mt][0] = c[mt][1] = c[mt][2] = c[mt][3] = 0.f;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const uint2 b = W[W_L2 + (j * 4 + s) * 32 + lane];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) mma16816(c[mt], a2[mt][s], b);
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            __half *r0 = tile + (16 * mt + g) * TILE_STRIDE + 16 + 8 * j + 2 * t;
            *reinterpret_cast<uint32_t *>(r0) = pack_h2(c[mt][0], c[mt][1]);
            *reinterpret_cast<uint32_t *>(r0 + 8 * TILE_STRIDE) = pack_h2(c[mt][2], c[mt][3]);
        }
    }
    __syncwarp();
}

/* Color head on the 32 rows: input tile cols 16..47 (density-network
 * outputs | SH), layer 3 (64 x 32 + bias from the 1-padding, ReLU),
 * [layer 4 (64 x 64, ReLU)], layer 5 (16 x 64).  Returns for each lane the
 * logits of rows (g, g+8) and (16+g, 24+g) at cols 2t, 2t+1 in out[mt][4]. */
template <int HEAD_HIDDEN>
__device__ __forceinline__ void color_mlp(const __half *tile, const uint2 *__restrict__ W, const float *__restrict__ bias3,
                                          int lane, float (&out)[2][4])
{
    const int t = lane & 3;
    uint32_t a3[2][2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int s = 0; s < 2; ++s) load_a(tile, mt, 16 + 16 * s, lane, a3[mt][s]);
    uint32_t a4[2][4][4];
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
        float c[2][2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float b0 = bias3[8 * (2 * jp + h) + 2 * t], b1 = bias3[8 * (2 * jp + h) + 2 * t + 1];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) { c[mt][h][0] = b0; c[mt][h][1] = b1; c[mt][h][2] = b0; c[mt][h][3] = b1; }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const uint2 b = W[W_L3 + ((2 * jp + h) * 2 + s) * 32 + lane];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) mma16816(c[mt][h], a3[mt][s], b);
            }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            a4[mt][jp][0] = pack_h2(fmaxf(c[mt][0][0], 0.f), fmaxf(c[mt][0][1], 0.f));
            a4[mt][jp][1] = pack_h2(fmaxf(c[mt][0][2], 0.f), fmaxf(c[mt][0][3], 0.f));
            a4[mt][jp][2] = pack_h2(fmaxf(c[mt][1][0], 0.f), fmaxf(c[mt][1][1], 0.f));
            a4[mt][jp][3] = pack_h2(fmaxf(c[mt][1][2], 0.f), fmaxf(c[mt][1][3], 0.f));
        }
    }
    if (HEAD_HIDDEN == 2) {
        uint32_t a5[2][4][4];
#pragma unroll
        for (int jp = 0; jp < 4; ++jp) {
            float c[2][2][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int h = 0; h < 2; ++h) c[mt][h][0] = c[mt][h][1] = c[mt][h][2] = c[mt][h][3] = 0.f;
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const uint2 b = W[W_L4 + ((2 * jp + h) * 4 + s) * 32 + lane];
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) mma16816(c[mt][h], a4[mt][s], b);
                }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                a5[mt][jp][0] = pack_h2(fmaxf(c[mt][0][0], 0.f), fmaxf(c[mt][0][1], 0.f));
                a5[mt][jp][1] = pack_h2(fmaxf(c[mt][0][2], 0.f), fmaxf(c[mt][0][3], 0.f));
                a5[mt][jp][2] = pack_h2(fmaxf(c[mt][1][0], 0.f), fmaxf(c[mt][1][1], 0.f));
                a5[mt][jp][3] = pack_h2(fmaxf(c[mt][1][2], 0.f), fmaxf(c[mt][1][3], 0.f));
            }
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int s = 0; s < 4; ++s)
#pragma unroll
                for (int q = 0; q < 4; ++q) a4[mt][s][q] = a5[mt][s][q];
    }
    /* layer 5: outputs 0..7 (only 0..2 used) */
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) out[mt][0] = out[mt][1] = out[mt][2] = out[mt][3] = 0.f;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const uint2 b = W[W_L5 + (0 * 4 + s) * 32 + lane];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) mma16816(out[mt], a4[mt][s], b);
    }
}

}  // namespace fvc
