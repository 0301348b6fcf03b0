/*
 * fvc_render.cu - the renderer as a wavefront of small kernels per
 * sub-iteration (PerformanceRenderer::render, src/performance_renderer.cu:
 * 214-286, and CachePerformanceRenderer::render,
 * src/cache_performance_renderer.cu:1059-1263):
 *
 *   raygen      one thread per pixel: generateRay + AABB clip; rays that hit
 *               enter the alive list (initRayPayloads_split_kernel,
 *               src/renderer.cu:86-134), the others are written out white.
 *   march       one thread per alive ray: up to S occupied samples
 *               (S = clamp(capacity / alive, 1, 8) as the reference's
 *               n_steps), appended as compacted rows; in the cached render
 *               each sample is classified (resample / cache / known empty)
 *               (sample_performance_kernel :15-69,
 *               sample_cache_performance_kernel :22-177).
 *   net_*       one warp per 32 rows: hash grid + density net + color head
 *               (resample rows) or trilinear cache lookup + color head (cache
 *               rows) on the tensor cores (NerfNetwork::inference /
 *               inferenceHead, generateNetworkInput_cache_shfl_perf_kernel_cg).
 *   composite   one thread per alive ray: the ray's rows merged by t0 and
 *               composited front to back with early termination; finished
 *               rays are written out, the others compacted into the next
 *               alive list (accumulate_performance_kernel :71-125,
 *               accumulate_cache_perf_kernel :789-908,
 *               compactPayloads_split_kernel src/renderer.cu:158-189).
 *
 * Counts live in device memory, so no kernel needs a host round trip; the
 * host reads the alive count every few sub-iterations to stop the loop.
 */
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <vector>

#include "fvc_kernels.h"

#include <cuda_fp16.h>

namespace fvc {

constexpr unsigned FULLMASK = 0xffffffffu;
constexpr int S_ROWS = 16;        /* rows per ray and sub-iteration (the reference keeps up to 8) */
static_assert(S_ROWS < 256, "the compositing kernel counts a ray's rows per miss reason in 8-bit fields");
constexpr int NET_WARPS = 8;
/* tcgen05 network kernel: CTAs resident per SM (launch bound and grid) and
 * hash levels whose gathers are in flight together.  Measured at 1080p on the
 * 3-cascade scene (resample-kernel ms per frame, plain / cached path):
 * 6 CTAs + groups of 2 (80 registers, spills) 37.2 / 34.5; 5 + 2: 30.0 / 22.5;
 * 5 + 4 (96 registers): 29.1 / 22.1; 4 + 4: 30.6 / 22.6. */
#ifndef FVC_TC_CTAS_PER_SM
#define FVC_TC_CTAS_PER_SM 5
#endif
#ifndef FVC_TC_HASH_GROUP
#define FVC_TC_HASH_GROUP 4
#endif

__device__ __forceinline__ unsigned lane_lt() { unsigned m; asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m)); return m; }
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

/* warp-aggregated atomicAdd: every active lane gets its offset */
__device__ __forceinline__ int warp_alloc(int *ctr, int n)
{
    const unsigned act = __activemask();
    int incl = n;
    const int lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(act, incl, o);
        if (lane >= o && ((act >> (lane - o)) & 1u)) incl += v;
    }
    /* the above scan is valid only for a full warp; fall back to per-lane atomics otherwise */
    if (act != FULLMASK) return atomicAdd(ctr, n);
    const int total = __shfl_sync(FULLMASK, incl, 31);
    int base = 0;
    if (lane == 31) base = atomicAdd(ctr, total);
    base = __shfl_sync(FULLMASK, base, 31);
    return base + incl - n;
}

/* compensated (Kahan) summation: sum += v with the running error in c */
__device__ __forceinline__ void kahan_add(float &sum, float &c, float v)
{
    const float y = __fsub_rn(v, c);
    const float t = __fadd_rn(sum, y);
    c = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

__device__ __forceinline__ void write_pixel(const RenderParams &p, int id, float4 acc, int4 counts)
{
    if (p.results) p.results[id] = acc;
    if (p.ray_counts) p.ray_counts[id] = counts;
    if (p.image) {
        /* writeImageBuffer_performance_kernel, src/performance_renderer.cu:127-149 */
        float cr = acc.x + acc.w, cg = acc.y + acc.w, cb = acc.z + acc.w;
        if (p.sample_index > 0) {
            const uchar4 prev = p.image[id];
            const float si = (float)p.sample_index;
            cr = (cr + (float)prev.x / 255.f * si) / (si + 1.f);
            cg = (cg + (float)prev.y / 255.f * si) / (si + 1.f);
            cb = (cb + (float)prev.z / 255.f * si) / (si + 1.f);
        }
        uchar4 o;
        o.x = (unsigned char)min(255, max(0, (int)(cr * 256.f)));
        o.y = (unsigned char)min(255, max(0, (int)(cg * 256.f)));
        o.z = (unsigned char)min(255, max(0, (int)(cb * 256.f)));
        o.w = 255;
        p.image[id] = o;
    }
}

/* ------------------------------------------------------------------------- */
/* raygen                                                                    */
/* ------------------------------------------------------------------------- */
/* the ray's first t1 (initRayPayloads_split_kernel, src/renderer.cu:119-124):
 * valid_t_from_t of the box entry plus, when not deterministic, the first
 * step times ld_random_t_offset(sample_index, ray_id * 56924617) */
__device__ __forceinline__ float start_t1(const DevCam &c, const DevSteps &st, float tn, int ray_id)
{
    const float start = valid_t_from_t(st, tn);
    const float toff = c.nd ? fvc_smp::t_offset((uint32_t)c.sample_index, (uint32_t)ray_id) : 0.0f;
    return F_ADD(start, F_MUL(calc_step(st, start), toff));
}

/* Pixels are visited in 8x4 tiles per warp so that a warp's rays are
 * neighbours (coherent marching and gathers). */
__global__ void __launch_bounds__(256) wf_raygen_kernel(RenderParams p)
{
    const int W = p.cam.W, H = p.cam.H;
    const int tiles_x = (W + 7) / 8, tiles_y = (H + 3) / 4;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int tile = gid >> 5, lane = lane_id();
    if (tile >= tiles_x * tiles_y) return;
    const int x = (tile % tiles_x) * 8 + (lane & 7), y = (tile / tiles_x) * 4 + (lane >> 3);
    const bool valid = x < W && y < H;
    bool hits = false;
    float3 o = make_float3(0, 0, 0), d = make_float3(0, 0, 0);
    float tn = 0.f, tf = 0.f;
    if (valid) {
        generate_ray_rm(p.cam, x, y, o, d);
        hits = ray_aabb(o, d, p.scene.aabb_from, p.scene.aabb_to, tn, tf);
    }
    const int id = y * W + x;
    if (valid && !hits) write_pixel(p, id, make_float4(0.f, 0.f, 0.f, 1.f), make_int4(0, 0, 0, 0));
    const unsigned m = __ballot_sync(FULLMASK, hits);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(p.counters + 0, __popc(m));
    base = __shfl_sync(FULLMASK, base, 0);
    if (hits) {
        RayState st;
        st.of = make_float4(o.x, o.y, o.z, fminf(tf, p.steps.far_));
        st.dt = make_float4(d.x, d.y, d.z, start_t1(p.cam, p.steps, tn, id));
        st.acc = make_float4(0.f, 0.f, 0.f, 1.f);
        st.comp = make_float4(0.f, 0.f, 0.f, 0.f);
        st.cnt = make_int4(id, 0, 0, 0);
        st.cnt2 = make_int4(0, 0, 0, 0);
        p.states[0][base + __popc(m & lane_lt())] = st;
    }
}

/* rays for a list of pixels (differentiable render): ray id = list index,
 * results[id] is written for rays that miss the scene box */
__global__ void __launch_bounds__(256) wf_raygen_list_kernel(RenderParams p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int W = p.cam.W, H = p.cam.H;
    const int pix = i < p.n_list ? p.pixel_list[i] : -1;
    const bool valid = pix >= 0 && pix < W * H;
    bool hits = false;
    float3 o = make_float3(0, 0, 0), d = make_float3(0, 0, 0);
    float tn = 0.f, tf = 0.f;
    if (valid) {
        generate_ray_rm(p.cam, pix % W, pix / W, o, d);
        hits = ray_aabb(o, d, p.scene.aabb_from, p.scene.aabb_to, tn, tf);
    }
    if (i < p.n_list && !hits) write_pixel(p, i, make_float4(0.f, 0.f, 0.f, 1.f), make_int4(0, 0, 0, 0));
    const unsigned m = __ballot_sync(FULLMASK, hits);
    int base = 0;
    if (lane_id() == 0 && m) base = atomicAdd(p.counters + 0, __popc(m));
    base = __shfl_sync(FULLMASK, base, 0);
    if (hits) {
        RayState st;
        st.of = make_float4(o.x, o.y, o.z, fminf(tf, p.steps.far_));
        st.dt = make_float4(d.x, d.y, d.z, start_t1(p.cam, p.steps, tn, pix));
        st.acc = make_float4(0.f, 0.f, 0.f, 1.f);
        st.comp = make_float4(0.f, 0.f, 0.f, 0.f);
        st.cnt = make_int4(i, 0, 0, 0);
        st.cnt2 = make_int4(0, 0, 0, 0);
        p.states[0][base + __popc(m & lane_lt())] = st;
    }
}

/* rays of a batch of views (one thread per pixel of the concatenated views) */
__global__ void __launch_bounds__(256) wf_raygen_views_kernel(RenderParams p)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.view_off[p.n_views];
    const bool valid = i < n;
    bool hits = false;
    float3 o = make_float3(0, 0, 0), d = make_float3(0, 0, 0);
    float tn = 0.f, tf = 0.f;
    int view = 0, local = 0;
    if (valid) {
        int lo = 0, hi = p.n_views - 1; /* the view holding ray i: last offset <= i */
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (p.view_off[mid] <= i) lo = mid; else hi = mid - 1;
        }
        view = lo;
        const DevCam &cam = p.views[lo];
        local = i - p.view_off[lo];
        generate_ray_rm(cam, local % cam.W, local / cam.W, o, d);
        hits = ray_aabb(o, d, p.scene.aabb_from, p.scene.aabb_to, tn, tf);
    }
    if (valid && !hits) write_pixel(p, i, make_float4(0.f, 0.f, 0.f, 1.f), make_int4(0, 0, 0, 0));
    const unsigned m = __ballot_sync(FULLMASK, hits);
    int base = 0;
    if (lane_id() == 0 && m) base = atomicAdd(p.counters + 0, __popc(m));
    base = __shfl_sync(FULLMASK, base, 0);
    if (hits) {
        RayState st;
        st.of = make_float4(o.x, o.y, o.z, fminf(tf, p.steps.far_));
        st.dt = make_float4(d.x, d.y, d.z, start_t1(p.views[view], p.steps, tn, local));
        st.acc = make_float4(0.f, 0.f, 0.f, 1.f);
        st.comp = make_float4(0.f, 0.f, 0.f, 0.f);
        st.cnt = make_int4(i, 0, 0, 0);
        st.cnt2 = make_int4(0, 0, 0, view);
        p.states[0][base + __popc(m & lane_lt())] = st;
    }
}

/* end of a graph-loop body (two sub-iterations): continue while rays are
 * alive and the iteration bound is not reached (guard bit 32 if it is) */
__global__ void wf_loop_cond_kernel(RenderParams p, cudaGraphConditionalHandle handle)
{
    const int iters = p.counters[5] + 2;
    p.counters[5] = iters;
    const bool alive = p.counters[0] > 0;
    if (alive && iters >= p.max_iterations) atomicOr(p.guard, 32);
    cudaGraphSetConditional(handle, (alive && iters < p.max_iterations) ? 1u : 0u);
}

/* ------------------------------------------------------------------------- */
/* march                                                                     */
/* ------------------------------------------------------------------------- */

/* Why a sample lies outside the cache's sampled region (REASON_*), or 0
 * when it lies inside: the frustum and known-range tests of
 * sample_cache_performance_kernel (src/cache_performance_renderer.cu:91-122),
 * which both cache renderers share, for the point c in the cache camera's
 * frame.  The sample is outside when any test fails; the reason named is the
 * first failing one in the order image, near plane, known range, froxel
 * depth.  The froxel depth (the step index of t, a logarithm) is computed
 * only for a sample that passes the first three.  fr receives the froxel
 * point (its z only past those tests), tfr the distance. */
__device__ __forceinline__ int unsampled_reason_at(const CacheView &C, const DevCam &ccam, const DevSteps &cst, float3 c, float3 &fr,
                                                   float &tfr)
{
    const float2 xy = cam2froxel_xy(c, ccam, tfr);
    fr = make_float3(xy.x, xy.y, 0.f);
    const bool in_fov = xy.x >= 0.f && xy.x < (float)C.fW && xy.y >= 0.f && xy.y < (float)C.fH;
    if (!in_fov) return REASON_OUTSIDE_FOV;
    const float kr = __ldg(C.known_ranges + (size_t)(int)floorf(xy.y) * C.fW + (int)floorf(xy.x));
    if (tfr < cst.near_) return REASON_BEFORE_NEAR;
    if (tfr > kr) return REASON_BEYOND_KNOWN;
    fr.z = froxel_z(cst, tfr, c.z);
    if (!(fr.z >= 0.f && fr.z < (float)C.fD)) return REASON_OUTSIDE_DEPTH;
    return REASON_NONE;
}

/* Classification of one occupied sample, sample_cache_performance_kernel
 * (src/cache_performance_renderer.cu:91-163): the row kind with its
 * REASON_* in the upper bits. */
__device__ __forceinline__ int classify(const RenderParams &p, const CacheView &C, const DevCam &ccam, const DevSteps &cst,
                                        float3 oc, float3 dc, float tm)
{
    float tfr;
    float3 fr;
    const int why = unsampled_reason_at(C, ccam, cst, at(oc, dc, tm), fr, tfr);
    if (why) return (p.render_mode == 1 ? KIND_SKIP : KIND_RESAMPLE) | (why << 2);
    if (p.render_mode == 2) return KIND_SKIP;
    const int bx = (int)F_MUL(fr.x, 0.125f), by = (int)F_MUL(fr.y, 0.125f), bz = (int)F_MUL(fr.z, 0.125f);
    const int packed = __ldg(C.packed_index + ((size_t)bz * C.bY + by) * C.bX + bx);
    if (packed < 0) return KIND_DROP | (REASON_BRICK_UNSET << 2);
    const float ax = F_ADD((float)(((packed >> 20) & 1023) * 8), F_SUB(fr.x, (float)(bx * 8)));
    const float ay = F_ADD((float)(((packed >> 10) & 1023) * 8), F_SUB(fr.y, (float)(by * 8)));
    const float az = F_ADD((float)((packed & 1023) * 8), F_SUB(fr.z, (float)(bz * 8)));
    const Voxel *v = texel(C, (int)floorf(ax), (int)floorf(ay), (int)floorf(az));
    if (!v || !(__ldg(&v->density) > 0.0f)) return KIND_DROP | (REASON_VOXEL_EMPTY << 2);
    return KIND_CACHE;
}

/* CacheBasicRenderer's per-sample decision and cache lookup
 * (sample_cache_kernel, src/cache_basic_renderer.cu:20-210; froxel2data and
 * fetchBrickTex3DInterpol, include/raymarch_common.h:331-444), all at the
 * sample's midpoint tm in the cache's froxel grid:
 *   - outside the frustum or the known range: resample;
 *   - brick without a slot, or the voxel under the point not set: dropped;
 *   - else the isset weight, the density slot and the 8 latents are
 *     interpolated: within the data array when the interpolation is Linear
 *     and the point lies inside its brick (or inter-brick interpolation is
 *     off, which clamps the point into the brick), by nearest texel for
 *     Nearest, otherwise over the 8 froxel corners each fetched through its
 *     own brick with the interpolation function's weights (unset -> 0, no
 *     isset weighting);
 *   - the variant turns the interpolated slot (or latent 0) into density and
 *     alpha and rewrites latent 0 (log of the density for the
 *     *Intermediates variants); with reweight_intermediates the latents are
 *     divided by the interpolated isset, latent 0 first multiplied by it when
 *     disable_reweighting_first_intermediate is set;
 *   - a cache sample needs alpha > alpha_thre, else it is dropped.
 * The texture unit's 8-bit fixed-point weights are not emulated: weights are
 * full float. */
__device__ __forceinline__ void basic_corners_array(const CacheView &C, float3 dp, const Voxel *(&vp)[8], float (&w)[8])
{
    const float fx = F_SUB(dp.x, 0.5f), fy = F_SUB(dp.y, 0.5f), fz = F_SUB(dp.z, 0.5f);
    const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
    const float lx = F_SUB(fx, x0), ly = F_SUB(fy, y0), lz = F_SUB(fz, z0);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
        w[c] = (ox ? lx : 1.0f - lx) * (oy ? ly : 1.0f - ly) * (oz ? lz : 1.0f - lz);
        vp[c] = texel(C, (int)x0 + ox, (int)y0 + oy, (int)z0 + oz);
    }
}

__device__ __forceinline__ int classify_basic(const RenderParams &p, const CacheView &C, const DevCam &ccam, const DevSteps &cst,
                                              float3 oc, float3 dc, float tm, float dt, float (&lat)[8], float &density)
{
    float tfr;
    float3 fr;
    const int why = unsampled_reason_at(C, ccam, cst, at(oc, dc, tm), fr, tfr);
    if (why) return KIND_RESAMPLE | (why << 2);
    /* froxel2data */
    const int bx = (int)F_MUL(fr.x, 0.125f), by = (int)F_MUL(fr.y, 0.125f), bz = (int)F_MUL(fr.z, 0.125f);
    float ix = F_SUB(fr.x, (float)(bx * 8)), iy = F_SUB(fr.y, (float)(by * 8)), iz = F_SUB(fr.z, (float)(bz * 8));
    bool inside_brick = true;
    if (C.inter_brick) {
        inside_brick = ix >= 0.5f && ix < 7.5f && iy >= 0.5f && iy < 7.5f && iz >= 0.5f && iz < 7.5f;
    } else {
        ix = fminf(fmaxf(ix, 0.5f), 7.5f);
        iy = fminf(fmaxf(iy, 0.5f), 7.5f);
        iz = fminf(fmaxf(iz, 0.5f), 7.5f);
    }
    const int packed = __ldg(C.packed_index + ((size_t)bz * C.bY + by) * C.bX + bx);
    if (packed < 0) return KIND_DROP | (REASON_BRICK_UNSET << 2);
    const float3 dp = make_float3(F_ADD((float)(((packed >> 20) & 1023) * 8), ix), F_ADD((float)(((packed >> 10) & 1023) * 8), iy),
                                  F_ADD((float)((packed & 1023) * 8), iz));
    const Voxel *vc = texel(C, (int)floorf(dp.x), (int)floorf(dp.y), (int)floorf(dp.z));
    if (!vc || !(__ldg(&vc->isset) > 0.0f)) return KIND_DROP | (REASON_VOXEL_EMPTY << 2);
    /* fetchBrickTex3DInterpol for isset, the density slot and the latents */
    const Voxel *vp[8];
    float wc[8];
    if (C.interp == INTERP_NEAREST) {
#pragma unroll
        for (int c = 0; c < 8; ++c) { vp[c] = c == 0 ? vc : nullptr; wc[c] = c == 0 ? 1.0f : 0.0f; }
    } else if (C.interp == INTERP_LINEAR && inside_brick) {
        basic_corners_array(C, dp, vp, wc);
    } else {
        cache_corners(C, fr, vp, wc);
    }
    float weight = 0.f, dac = 0.f, ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (!vp[c]) continue;
        const float w = wc[c];
        float2 di;
        uint4 lt;
        ld_voxel(vp[c], di, lt);
        weight = fmaf(w, di.y, weight);
        dac = fmaf(w, di.x, dac);
        const uint32_t lw[4] = {lt.x, lt.y, lt.z, lt.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 fq = __half22float2(*reinterpret_cast<const __half2 *>(&lw[q]));
            ls[2 * q] = fmaf(w, fq.x, ls[2 * q]);
            ls[2 * q + 1] = fmaf(w, fq.y, ls[2 * q + 1]);
        }
    }
    float alpha;
    switch (C.variant) {
    case VARIANT_ALPHA:
        alpha = dac;
        density = -logf(fmaxf(1.0f - alpha, 1e-6f)) / dt;
        break;
    case VARIANT_INTERMEDIATES:
        density = expf(ls[0] / weight);
        alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-density * dt)));
        break;
    case VARIANT_DENSITY_INTERMEDIATES:
        density = ls[0];
        alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-density * dt)));
        ls[0] = logf(density);
        break;
    case VARIANT_ALPHA_INTERMEDIATES:
        alpha = ls[0];
        density = -logf(fmaxf(1.0f - alpha, 1e-6f)) / dt;
        ls[0] = logf(density);
        break;
    default: /* Density */
        density = dac;
        alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-density * dt)));
        break;
    }
    if (C.reweight && C.keep_first) ls[0] *= weight;
    if (!(alpha > p.scene.alpha_thre)) return KIND_DROP | (REASON_ALPHA << 2);
    const float div = C.reweight ? weight : 1.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) lat[j] = ls[j] / div;
    return KIND_CACHE;
}

/* Marches every alive ray a fixed number of steps (lanes stay converged),
 * keeping at most S_ROWS occupied samples; the samples become rows
 * (t0, alive slot) that are contiguous and in t order per ray.  The plain
 * renderer also contracts the sample position here; the cached renderer
 * classifies the rows in wf_classify_kernel. */
#ifndef FVC_RAY_BLOCKS_PER_SM
#define FVC_RAY_BLOCKS_PER_SM 64 /* blocks of 128 threads per SM for the per-ray kernels (march, composite): more
                                  * blocks than fit balance the rays' uneven work (1080p march: 16 -> 12.7 ms,
                                  * 32 -> 12.0, 64 -> 11.5, 128 -> 11.6) */
#endif

template <bool CACHED, bool FUSED = false>
__global__ void __launch_bounds__(128) wf_march_kernel(RenderParams p, int it)
{
    const int n_alive = p.counters[it & 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) p.counters[(it + 1) & 1] = 0; /* next alive count */
    /* samples per ray this sub-iteration: the compaction batch (row_target, else the row capacity)
     * over the alive rays, clamped to [1, S_ROWS] as n_steps_curr_subiter of
     * src/performance_renderer.cu:249 (the host keeps row_target <= row_capacity) */
    const int batch = p.row_target > 0 ? p.row_target : p.row_capacity;
    const int S = max(1, min(S_ROWS, batch / max(1, n_alive)));
    RayState *states = p.states[it & 1];
    for (int base = blockIdx.x * blockDim.x; base < n_alive; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool valid = i < n_alive;
        float t0s[S_ROWS];
        int n = 0, steps = 0;
        float4 of = make_float4(0, 0, 0, 0), dt4 = make_float4(0, 0, 0, 0);
        bool done = false;
        if (valid) {
            of = states[i].of;
            dt4 = states[i].dt;
            const float3 o = make_float3(of.x, of.y, of.z), d = make_float3(dt4.x, dt4.y, dt4.z);
            float t1 = dt4.w;
            /* empty-space skipping: steps whose midpoint lies before t_free are in an empty cell
             * (occupied_skip's conservative DDA bound) and skip the occupancy lookup; the step
             * sequence and every occupancy outcome stay those of the plain march */
            const float3 inv_d = make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
            float t_free = -1e30f;
            for (int c0 = 0; c0 < p.steps_per_iter; c0 += 4) {
                float t0c[4], t1c[4];
                bool past[4], occ[4];
                float tt = t1;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    t0c[c] = tt;
                    const float dtc = calc_step(p.steps, tt);
                    t1c[c] = F_ADD(tt, dtc);
                    const float tm = F_MUL(F_ADD(tt, t1c[c]), 0.5f);
                    past[c] = tm > of.w;
                    bool oc = false;
                    if (!past[c] && !(tm < t_free)) {
                        if (p.skip_empty) oc = occupied_skip(p.scene, p.bits, o, d, inv_d, tm, dtc, t_free);
                        else oc = occupied(p.scene, p.bits, at(o, d, tm));
                    }
                    occ[c] = oc;
                    tt = t1c[c];
                }
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if (!done && n < S) {
                        ++steps;
                        if (past[c]) {
                            done = true;
                        } else {
                            t1 = t1c[c];
                            if (occ[c]) t0s[n++] = t0c[c];
                        }
                    }
                }
                if (done || n >= S) break;
            }
            dt4.w = t1;
        }
        const int rbase = warp_alloc(p.counters + 2, n);
        int n_res = 0, n_hit = 0;
        uint32_t kinds = 0; /* FUSED: 2 bits per row, its kind */
        if (FUSED && valid) {
            /* the cached renderer's classification of this ray's rows (wf_classify_kernel's
             * non-basic form), with the ray moved into the cache camera once per ray */
            const ViewCache *vc = p.view_caches ? p.view_caches + states[i].cnt2.w : nullptr;
            const CacheView &C = vc ? vc->cache : p.cache;
            const DevCam &ccam = vc ? vc->ccam : p.ccam;
            const DevSteps &cst = vc ? vc->csteps : p.csteps;
            const float3 o = make_float3(of.x, of.y, of.z), d = make_float3(dt4.x, dt4.y, dt4.z);
            float3 oc, dc;
            transform_ray(ccam.w2c, o, d, oc, dc);
            for (int s = 0; s < n; ++s) {
                const float t0 = t0s[s];
                const float dt = calc_step(p.steps, t0);
                const float tm = F_MUL(F_ADD(t0, F_ADD(t0, dt)), 0.5f);
                const float tmh = F_ADD(t0, F_MUL(dt, 0.5f));
                const int code = classify(p, C, ccam, cst, oc, dc, tm);
                const int kind = row_kind_of(code);
                float4 pay = make_float4(0.f, 0.f, 0.f, 0.f);
                if (kind == KIND_RESAMPLE) {
                    const float3 pc = contract(p.scene, at(o, d, tmh));
                    pay = make_float4(pc.x, pc.y, pc.z, 0.f);
                    ++n_res;
                } else if (kind == KIND_CACHE) {
                    float tf2;
                    const float3 fr = cam2froxel(at(oc, dc, tmh), ccam, cst, tf2);
                    pay = make_float4(fr.x, fr.y, fr.z, 0.f);
                    ++n_hit;
                }
                p.row_t0[rbase + s] = t0;
                p.row_slot[rbase + s] = i;
                p.row_pay[rbase + s] = pay;
                p.row_kind[rbase + s] = (uint8_t)code;
                kinds |= (uint32_t)kind << (2 * s);
            }
        }
        if (FUSED) {
            /* the resample rows and the cache rows each go to a list, so that the network's tiles hold one
             * kind of row: a cache row never waits on its tile's hash gathers */
            int rb = warp_alloc(p.counters + 3, n_res), hb = warp_alloc(p.counters + 4, n_hit);
            for (int s = 0; s < n && (n_res | n_hit); ++s) {
                const uint32_t kind = (kinds >> (2 * s)) & 3u;
                if (kind == KIND_RESAMPLE) p.res_list[rb++] = rbase + s;
                else if (kind == KIND_CACHE) p.cache_list[hb++] = rbase + s;
            }
        }
        if (valid) {
            for (int s = 0; s < n && !FUSED; ++s) {
                p.row_t0[rbase + s] = t0s[s];
                p.row_slot[rbase + s] = i;
                if (!CACHED) {
                    /* sample_performance_kernel :52-58: midpoint (t0+t1)/2, contracted */
                    const float t0 = t0s[s];
                    const float tm = F_MUL(F_ADD(t0, F_ADD(t0, calc_step(p.steps, t0))), 0.5f);
                    const float3 pc = contract(p.scene, at(make_float3(of.x, of.y, of.z), make_float3(dt4.x, dt4.y, dt4.z), tm));
                    p.row_pay[rbase + s] = make_float4(pc.x, pc.y, pc.z, 0.f);
                }
            }
            p.ray_rows[i] = make_int2(rbase, n);
            states[i].dt = dt4;
            int4 c = states[i].cnt;
            c.w += steps;
            states[i].cnt = c;
            int4 c2 = states[i].cnt2;
            c2.y = done ? 1 : 0;
            c2.z += n;
            states[i].cnt2 = c2;
            if (p.max_samples_per_ray > 0 && c2.z > p.max_samples_per_ray) atomicOr(p.guard, 1);
        }
        const int ws = __reduce_add_sync(FULLMASK, steps);
        if (lane_id() == 0 && ws) atomicAdd(&p.stats->n_steps, (unsigned long long)ws);
    }
}

/* the cache a row's ray renders against: its view's cache in a batch, else the renderer's */
__device__ __forceinline__ const CacheView &row_cache(const RenderParams &p, const RayState *states, int r)
{
    return p.view_caches ? p.view_caches[states[p.row_slot[r]].cnt2.w].cache : p.cache;
}

/* Trilinear, isset-weighted lookup of the cache for one froxel point,
 * generateNetworkInput_cache_shfl_perf_kernel_cg
 * (src/cache_performance_renderer.cu:678-787): head input = log of the
 * interpolated density (not renormalised) and latents / interpolated isset. */
__device__ __forceinline__ void cache_lookup(const CacheView &C, float3 f, float &logd, float (&lat)[8])
{
    const Voxel *vp[8];
    float wc[8];
    cache_corners(C, f, vp, wc);
    float wsum = 0.f, dsum = 0.f, ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        if (!vp[c]) continue;
        const float w = wc[c];
        float2 di;
        uint4 lt;
        ld_voxel(vp[c], di, lt);
        wsum = fmaf(w, di.y, wsum);
        dsum = fmaf(w, di.x, dsum);
        const uint32_t lw[4] = {lt.x, lt.y, lt.z, lt.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 fq = __half22float2(*reinterpret_cast<const __half2 *>(&lw[q]));
            ls[2 * q] = fmaf(w, fq.x, ls[2 * q]);
            ls[2 * q + 1] = fmaf(w, fq.y, ls[2 * q + 1]);
        }
    }
    const float inv = 1.0f / wsum;
#pragma unroll
    for (int j = 0; j < 8; ++j) lat[j] = ls[j] * inv;
    if (C.first_latent_is_density) {
        /* DensityIntermediates (:776-781): latent 0 holds the density; the
         * head input is log(sum w density) * wsum / wsum, the other latents
         * are renormalised by the interpolated isset */
        lat[0] = __fdiv_rn(logf(ls[0]) * wsum, wsum);
        logd = lat[0];
    } else {
        logd = logf(fmaxf(dsum, 1e-6f));
    }
}

/* One thread per row of the cached render: classification
 * (sample_cache_performance_kernel :91-163) and the network input of the
 * row (generateNetworkInput_resample_perf_kernel :231-238 /
 * _preparation_perf_kernel :284-297 evaluate it at t0 + dt/2): the
 * contracted position of a resample row, the trilinear cache lookup of a
 * cache row (its 8 head inputs from K = latent_offset go to row_lat at the
 * row's place in the cache list, its log-density to the high half of
 * row_out.y; the froxel point stays in row_pay for the adjoint); appends
 * the row id to the resample or cache list. */
/* the initial view direction of a cache row for a view-dependent head: from
 * the cache camera to the sample, unit_to_01; the head reads it from the row
 * payload */
__device__ __forceinline__ float3 cache_viewdir01(float3 wp, const DevCam &ccam)
{
    const float vx = wp.x - ccam.c2w[3], vy = wp.y - ccam.c2w[7], vz = wp.z - ccam.c2w[11];
    const float inv = rsqrtf(vx * vx + vy * vy + vz * vz);
    return make_float3((vx * inv + 1.0f) / 2.0f, (vy * inv + 1.0f) / 2.0f, (vz * inv + 1.0f) / 2.0f);
}

template <bool VD>
__global__ void __launch_bounds__(256) wf_classify_kernel(RenderParams p, int it)
{
    const int n_rows = p.counters[2];
    const RayState *states = p.states[it & 1];
    for (int base = blockIdx.x * blockDim.x; base < n_rows; base += gridDim.x * blockDim.x) {
        const int r = base + threadIdx.x;
        int kind = KIND_SKIP, code = KIND_SKIP;
        float logd = 0.f, lat[8];
        if (r < n_rows) {
            const int slot = p.row_slot[r];
            const float t0 = p.row_t0[r];
            const float4 of = states[slot].of, dt4 = states[slot].dt;
            const float3 o = make_float3(of.x, of.y, of.z), d = make_float3(dt4.x, dt4.y, dt4.z);
            const ViewCache *vc = p.view_caches ? p.view_caches + states[slot].cnt2.w : nullptr;
            const CacheView &C = vc ? vc->cache : p.cache;
            const DevCam &ccam = vc ? vc->ccam : p.ccam;
            const DevSteps &cst = vc ? vc->csteps : p.csteps;
            float3 oc, dc;
            transform_ray(ccam.w2c, o, d, oc, dc);
            const float dt = calc_step(p.steps, t0);
            const float tm = F_MUL(F_ADD(t0, F_ADD(t0, dt)), 0.5f);
            if (p.basic_cache) {
                /* CacheBasicRenderer: lookup and resample position at the midpoint;
                 * a cache row keeps its looked-up density for compositing */
                float density = 0.f;
                code = classify_basic(p, C, ccam, cst, oc, dc, tm, dt, lat, density);
                kind = row_kind_of(code);
                if (kind == KIND_RESAMPLE) {
                    const float3 pc = contract(p.scene, at(o, d, tm));
                    p.row_pay[r] = make_float4(pc.x, pc.y, pc.z, 0.f);
                } else if (kind == KIND_CACHE) {
                    float3 iv = make_float3(0.f, 0.f, 0.f);
                    if (VD) iv = cache_viewdir01(at(o, d, tm), ccam); /* src/cache_basic_renderer.cu:86-87,198 */
                    p.row_pay[r] = make_float4(iv.x, iv.y, iv.z, density);
                    logd = logf(density);
                }
            } else {
                const float tmh = F_ADD(t0, F_MUL(dt, 0.5f));
                code = classify(p, C, ccam, cst, oc, dc, tm);
                kind = row_kind_of(code);
                if (kind == KIND_RESAMPLE) {
                    const float3 pc = contract(p.scene, at(o, d, tmh));
                    p.row_pay[r] = make_float4(pc.x, pc.y, pc.z, 0.f);
                } else if (kind == KIND_CACHE) {
                    float tf2;
                    const float3 fr = cam2froxel(at(oc, dc, tmh), ccam, cst, tf2);
                    p.row_pay[r] = make_float4(fr.x, fr.y, fr.z, 0.f);
                    cache_lookup(C, fr, logd, lat);
                    if (VD) { /* src/cache_performance_renderer.cu:290-312 */
                        const float3 iv = cache_viewdir01(at(o, d, tmh), ccam);
                        p.row_pay[r] = make_float4(iv.x, iv.y, iv.z, 0.f);
                    }
                }
            }
            p.row_kind[r] = (uint8_t)code;
        }
        const unsigned m0 = __ballot_sync(FULLMASK, kind == KIND_RESAMPLE), m1 = __ballot_sync(FULLMASK, kind == KIND_CACHE);
        int b0 = 0, b1 = 0;
        if (lane_id() == 0) {
            if (m0) b0 = atomicAdd(p.counters + 3, __popc(m0));
            if (m1) b1 = atomicAdd(p.counters + 4, __popc(m1));
        }
        b0 = __shfl_sync(FULLMASK, b0, 0);
        b1 = __shfl_sync(FULLMASK, b1, 0);
        if (kind == KIND_RESAMPLE) p.res_list[b0 + __popc(m0 & lane_lt())] = r;
        if (kind == KIND_CACHE) {
            const int kc = b1 + __popc(m1 & lane_lt());
            p.cache_list[kc] = r;
            p.row_lat[kc] = make_uint4(pack_h2(lat[0], lat[1]), pack_h2(lat[2], lat[3]), pack_h2(lat[4], lat[5]), pack_h2(lat[6], lat[7]));
            p.row_out[r] = make_uint2(0u, (uint32_t)__half_as_ushort(__float2half_rn(logd)) << 16);
        }
    }
}

/* The cache rows' trilinear lookups of a sub-iteration classified in the
 * march (cache_lookup at the froxel point in the row payload), one thread
 * per row of the cache list, at full occupancy so that many rows' eight
 * corner gathers are in flight at once.  The head input goes to row_lat at
 * the row's own index and its fp16 log-density to the high half of
 * row_out.y, which the network kernel's MODE 2 reads for a cache row. */
__global__ void __launch_bounds__(256) wf_cache_lookup_kernel(RenderParams p, int it)
{
    const int n_rows = p.counters[4];
    const RayState *states = p.states[it & 1];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_rows; k += gridDim.x * blockDim.x) {
        const int r = p.cache_list[k];
        const float4 fr = p.row_pay[r];
        float logd, lat[8];
        cache_lookup(row_cache(p, states, r), make_float3(fr.x, fr.y, fr.z), logd, lat);
        p.row_lat[r] = make_uint4(pack_h2(lat[0], lat[1]), pack_h2(lat[2], lat[3]), pack_h2(lat[4], lat[5]), pack_h2(lat[6], lat[7]));
        p.row_out[r] = make_uint2(0u, (uint32_t)__half_as_ushort(__float2half_rn(logd)) << 16);
    }
}

/* the view-dependent form only for those models: the default one keeps its
 * register count (and so its occupancy) */
static inline void launch_classify(const RenderParams &p, int it, int n_sms, cudaStream_t s)
{
    if (p.view_dependent) wf_classify_kernel<true><<<n_sms * 8, 256, 0, s>>>(p, it);
    else wf_classify_kernel<false><<<n_sms * 8, 256, 0, s>>>(p, it);
}

/* ------------------------------------------------------------------------- */
/* network over rows                                                         */
/* ------------------------------------------------------------------------- */
struct NetSmem {
    uint2 W[W_TOTAL];
    float bias3[64];
    __half tile[NET_WARPS][32 * TILE_STRIDE];
};

__device__ __forceinline__ void store_logits(__half *tile, const float (&lo)[2][4], int lane)
{
    const int g = lane >> 2, t = lane & 3;
    if (t < 2) {
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            __half *r0 = tile + (16 * mt + g) * TILE_STRIDE + 48 + 2 * t;
            *reinterpret_cast<uint32_t *>(r0) = pack_h2(lo[mt][0], lo[mt][1]);
            *reinterpret_cast<uint32_t *>(r0 + 8 * TILE_STRIDE) = pack_h2(lo[mt][2], lo[mt][3]);
        }
    }
}

__device__ __forceinline__ float3 dir01_of(const RayState *states, int slot)
{
    const float4 d = states[slot].dt;
    return make_float3(F_MUL(F_ADD(d.x, 1.0f), 0.5f), F_MUL(F_ADD(d.y, 1.0f), 0.5f), F_MUL(F_ADD(d.z, 1.0f), 0.5f)); /* / 2, exact */
}

/* Network over the resample rows (all rows of the plain renderer). */
template <int HEAD_HIDDEN, bool LIST>
__global__ void __launch_bounds__(NET_WARPS * 32, 2) wf_net_resample_kernel(RenderParams p, int it)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    NetSmem &S = *reinterpret_cast<NetSmem *>(smem_raw);
    const int n_rows = LIST ? p.counters[3] : p.counters[2];
    if (n_rows == 0) return;
    for (int i = threadIdx.x; i < W_TOTAL; i += blockDim.x) S.W[i] = p.weights[i];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) S.bias3[i] = p.bias3[i];
    __syncthreads();
    const int lane = lane_id(), w = threadIdx.x >> 5;
    __half *tile = S.tile[w];
    __half *trow = tile + lane * TILE_STRIDE;
    const RayState *states = p.states[it & 1];
    const int n_batches = (n_rows + 31) / 32;
    for (int b = blockIdx.x * NET_WARPS + w; b < n_batches; b += gridDim.x * NET_WARPS) {
        const int k = b * 32 + lane;
        const int r = k < n_rows ? (LIST ? p.res_list[k] : k) : -1;
        if (r >= 0) {
            const float4 pw = p.row_pay[r];
            hash_encode(p.grid, p.table, make_float3(pw.x, pw.y, pw.z), reinterpret_cast<__half2 *>(trow));
            sh16(dir01_of(states, p.row_slot[r]), reinterpret_cast<__half2 *>(trow + 32));
        } else {
#pragma unroll
            for (int c = 0; c < 24; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
        }
        __syncwarp();
        density_mlp(tile, S.W, lane);
        float lo[2][4];
        color_mlp<HEAD_HIDDEN>(tile, S.W, S.bias3, lane, lo);
        store_logits(tile, lo, lane);
        __syncwarp();
        if (r >= 0) {
            const uint32_t rg = *reinterpret_cast<const uint32_t *>(trow + 48);
            const uint32_t bs = (uint32_t)__half_as_ushort(trow[50]) | ((uint32_t)__half_as_ushort(trow[16]) << 16);
            p.row_out[r] = make_uint2(rg, bs);
        }
        __syncwarp();
    }
}

/* the head input of cache row r (place k in the cache list) as
 * classification looked it up: halves 16..31
 * of trow (log-density at 16 when latent_offset is 1, the latents from
 * 16 + latent_offset, zeros after) */
/* the head input (16 fp16 after the density layer's place: log-density at
 * K = 0 when latent_offset is 1, the 8 latents from K = latent_offset) of a
 * cache row from its lookup */
__device__ __forceinline__ void cache_head_input(uint4 lt, uint32_t ld, int latent_offset, uint32_t (&h)[8])
{
    if (latent_offset == 0) {
        h[0] = lt.x; h[1] = lt.y; h[2] = lt.z; h[3] = lt.w;
        h[4] = h[5] = h[6] = h[7] = 0u;
    } else {
        h[0] = ld | (lt.x << 16);
        h[1] = (lt.x >> 16) | (lt.y << 16);
        h[2] = (lt.y >> 16) | (lt.z << 16);
        h[3] = (lt.z >> 16) | (lt.w << 16);
        h[4] = lt.w >> 16;
        h[5] = h[6] = h[7] = 0u;
    }
}

__device__ __forceinline__ void cache_row_input(const RenderParams &p, int k, int r, __half *trow)
{
    uint32_t h[8];
    cache_head_input(p.row_lat[k], p.row_out[r].y >> 16, p.latent_offset, h);
    uint32_t *o = reinterpret_cast<uint32_t *>(trow + 16);
#pragma unroll
    for (int q = 0; q < 8; ++q) o[q] = h[q];
}

template <int HEAD_HIDDEN>
__global__ void __launch_bounds__(NET_WARPS * 32, 2) wf_net_cache_kernel(RenderParams p, int it)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    NetSmem &S = *reinterpret_cast<NetSmem *>(smem_raw);
    const int n_rows = p.counters[4];
    if (n_rows == 0) return;
    for (int i = threadIdx.x; i < W_TOTAL; i += blockDim.x) S.W[i] = p.weights[i];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) S.bias3[i] = p.bias3[i];
    __syncthreads();
    const int lane = lane_id(), w = threadIdx.x >> 5;
    __half *tile = S.tile[w];
    __half *trow = tile + lane * TILE_STRIDE;
    const RayState *states = p.states[it & 1];
    const int n_batches = (n_rows + 31) / 32;
    for (int b = blockIdx.x * NET_WARPS + w; b < n_batches; b += gridDim.x * NET_WARPS) {
        const int k = b * 32 + lane;
        const int r = k < n_rows ? p.cache_list[k] : -1;
        if (r >= 0) {
            cache_row_input(p, k, r, trow);
            sh16(dir01_of(states, p.row_slot[r]), reinterpret_cast<__half2 *>(trow + 32));
        } else {
#pragma unroll
            for (int c = 8; c < 24; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
        }
        __syncwarp();
        float lo[2][4];
        color_mlp<HEAD_HIDDEN>(tile, S.W, S.bias3, lane, lo);
        store_logits(tile, lo, lane);
        __syncwarp();
        if (r >= 0) {
            const uint32_t rg = *reinterpret_cast<const uint32_t *>(trow + 48);
            const uint32_t bs = (uint32_t)__half_as_ushort(trow[50]) | ((uint32_t)__half_as_ushort(trow[16]) << 16);
            p.row_out[r] = make_uint2(rg, bs);
        }
        __syncwarp();
    }
}

/* ------------------------------------------------------------------------- */
/* network over rows on the 5th-generation tensor cores                      */
/* ------------------------------------------------------------------------- */
/* One CTA of 128 threads per 128-row tile; thread t owns row t and TMEM lane
 * t.  The activations of a tile live in ONE shared-memory tile in the
 * canonical K-major layout that each layer overwrites in place (a layer's
 * epilogue runs only after its MMA has finished reading the tile); weights
 * stay resident in shared memory; accumulators use 64 TMEM columns (hidden
 * layers in cols 0..63, the 16-wide output layers in cols 0..15 once the
 * previous accumulator has been read).  37 KB of shared memory and 64
 * columns per CTA; FVC_TC_CTAS_PER_SM of them share an SM.  One thread issues each layer's MMAs and
 * commits them to an mbarrier; the CTA waits (bounded), reads its rows back
 * with tcgen05.ld, applies ReLU / fp16 rounding and writes the next layer's
 * operand. */
struct __align__(128) TcSmem {
    uint8_t X[128 * 64 * 2];
    float bias3[64];
    uint64_t mbar;
    uint32_t tmem_base;
    /* the weight tiles, last: a head with the frequency encoding (TCF_WBYTES) launches with the extra
     * bytes past the struct (tc_smem_bytes), the others keep the smaller footprint, so that 5 CTAs
     * leave the SM its larger L1 share for the hash gathers */
    __align__(128) uint8_t W[TC_WBYTES];
};
/* dynamic shared memory of a TcSmem launch */
static inline size_t tc_smem_bytes(int freq) { return sizeof(TcSmem) + (freq ? (size_t)(TCF_WBYTES - TC_WBYTES) : 0); }

constexpr long long TC_WAIT_LIMIT = 2000000000ll; /* ~1 s of SM clocks */
constexpr int TC_COLS = 64;
static_assert(FVC_TC_CTAS_PER_SM * TC_COLS <= 512, "resident CTAs must fit in the SM's 512 TMEM columns");

/* row `row`'s 8 fp16 values of K-chunk c of a tile with K columns */
__device__ __forceinline__ void st_chunk(uint8_t *tile, int row, int c, int K, uint4 v)
{
    *reinterpret_cast<uint4 *>(tile + kmajor_offset(row, 8 * c, K)) = v;
}

__device__ __forceinline__ uint4 pack8(const float *v)
{
    return make_uint4(pack_h2(v[0], v[1]), pack_h2(v[2], v[3]), pack_h2(v[4], v[5]), pack_h2(v[6], v[7]));
}

/* issue one layer: D[tmem_col] = A (128 x K, tile at a) * B^T (N x K, tile at b) */
__device__ __forceinline__ void tc_layer(uint32_t tmem, const uint8_t *a, const uint8_t *b, int K, int N)
{
    const uint32_t sbo = (uint32_t)(K / 8) * 128u;
    const uint32_t id = idesc_f16(128, N, false);
    const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
    for (int kc = 0; kc < K / 16; ++kc)
        tc_mma_f16(tmem, umma_desc(a0 + 256u * kc, 128u, sbo), umma_desc(b0 + 256u * kc, 128u, sbo), id, kc > 0 ? 1u : 0u);
}

/* 64 accumulator columns of this thread's row -> (+bias) ReLU -> fp16 row of
 * a K=64 tile.  The bias is added in fp32 (packed f32x2), and the ReLU runs on
 * the rounded half2 pairs: rounding is monotonic and maps 0 to 0, and
 * __hmax2, like fmaxf, returns the non-NaN operand and prefers +0, so the
 * bits equal fmaxf-then-round with one instruction per pair instead of two. */
__device__ __forceinline__ void epi_hidden(uint32_t taddr, const float *bias, uint8_t *dst, int row)
{
    const __half2 zero = __float2half2_rn(0.0f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float v[32];
        tmem_ld32(taddr + 32 * h, v);
        tmem_wait_ld();
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            float2 x = make_float2(v[2 * i], v[2 * i + 1]);
            if (bias) x = __fadd2_rn(x, make_float2(bias[32 * h + 2 * i], bias[32 * h + 2 * i + 1]));
            const __half2 r = __hmax2(__float22half2_rn(x), zero);
            w[i] = *reinterpret_cast<const uint32_t *>(&r);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) st_chunk(dst, row, 4 * h + q, 64, make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]));
    }
}

/* the MMAs of one layer, then the bounded wait for their completion */
__device__ __forceinline__ bool tc_run(TcSmem &S, uint32_t tmem, const uint8_t *b, int K, int N, uint32_t &phase)
{
    if (threadIdx.x == 0) {
        tc_fence_after();
        tc_layer(tmem, S.X, b, K, N);
        tc_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    tc_fence_after();
    return ok;
}

/* after a thread rewrote its row of the operand tile: make it visible to the
 * tensor core and order it after this thread's TMEM reads */
__device__ __forceinline__ bool tc_publish(bool ok)
{
    fence_proxy_async();
    tc_fence_before();
    return __syncthreads_or(!ok) == 0;
}

/* frequency_encoding (include/nerf_network.h:55-81) of one axis of the
 * network's input position: sin(pi 2^k x) for k < 4, then the cosines (the
 * reference's phase of pi/2), rounded to fp16; x 2^k is exact. */
__device__ __forceinline__ uint4 freq_chunk(float x)
{
    float v[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float xk = x * (float)(1 << k);
        v[k] = sinpif(xk);
        v[4 + k] = cospif(xk);
    }
    return pack8(v);
}

/* the head's input position of a cache row: the contracted point at the
 * midpoint the row's network input is evaluated at (t0 + dt/2,
 * generateNetworkInput_preparation_perf_kernel :284-297; (t0 + t1)/2 for the
 * basic cache renderer) */
__device__ __forceinline__ float3 cache_row_position(const RenderParams &p, const RayState *states, int r)
{
    const int slot = p.row_slot[r];
    const float4 of = states[slot].of, dt4 = states[slot].dt;
    const float t0 = p.row_t0[r], dt = calc_step(p.steps, t0);
    const float t = p.basic_cache ? F_MUL(F_ADD(t0, F_ADD(t0, dt)), 0.5f) : F_ADD(t0, F_MUL(dt, 0.5f));
    return contract(p.scene, at(make_float3(of.x, of.y, of.z), make_float3(dt4.x, dt4.y, dt4.z), t));
}

/* MODE 0: resample rows (the list, or all rows of the plain path); MODE 1: the
 * cache list (head only); MODE 2: both lists of a cached sub-iteration
 * classified by the march in one launch, the resample list's tiles first
 * (hash features, density layers, head), then the cache list's tiles (the
 * head input of each row's lookup, wf_cache_lookup_kernel; head only), so
 * that no tile mixes the two kinds of row. */
template <int MODE, int HH, bool LIST>
__global__ void __launch_bounds__(128, FVC_TC_CTAS_PER_SM) wf_net_tc_kernel(RenderParams p, int it)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
    const int n_rows = MODE == 0 ? (LIST ? p.counters[3] : p.counters[2]) : MODE == 1 ? p.counters[4] : p.counters[3];
    const int n_hit = MODE == 2 ? p.counters[4] : 0;
    if (n_rows == 0 && n_hit == 0) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    /* the weights arrive by one bulk copy on the TMA engine, completing the
     * mbarrier's phase 0; the layers' MMA commits complete the later phases */
    /* the head's input width and tile layout: 32 inputs (TC_*), or 64 with the frequency encoding (TCF_*) */
    const int HK = p.freq ? 64 : 32;
    const int wb3 = p.freq ? TCF_B3 : TC_B3, wb4 = p.freq ? TCF_B4 : TC_B4, wb5 = p.freq ? TCF_B5 : TC_B5;
    if (tid == 0) {
        const int wbytes = p.freq ? TCF_WBYTES : TC_WBYTES;
        mbar_init(&S.mbar, 1);
        mbar_arrive_expect_tx(&S.mbar, wbytes);
        bulk_copy_g2s(S.W, p.weights_tc, wbytes, &S.mbar);
    }
    if (tid < 64) S.bias3[tid] = p.bias3[tid];
    if (warp == 0) tmem_alloc(&S.tmem_base, TC_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const RayState *states = p.states[it & 1];
    uint32_t phase = 0;
    bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    const int res_tiles = (n_rows + 127) / 128;
    const int n_tiles = res_tiles + (n_hit + 127) / 128;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        int k = tile * 128 + tid, r = -1, kind = KIND_RESAMPLE;
        if (MODE == 2 && tile >= res_tiles) {
            k = (tile - res_tiles) * 128 + tid;
            kind = KIND_CACHE;
            r = k < n_hit ? p.cache_list[k] : -1;
        } else {
            r = k < n_rows ? (MODE == 0 ? (LIST ? p.res_list[k] : k) : MODE == 1 ? p.cache_list[k] : p.res_list[k]) : -1;
        }
        __half2 sh[8];
        uint16_t log_density = 0;
        if (r >= 0) sh16(dir01_of(states, p.row_slot[r]), sh);
        else for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
        if (MODE != 1) {
            /* ---- hash features -> tile (K = 32); MODE 2 cache rows: the cache lookup ---- */
            __half2 feat[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) feat[q] = __floats2half2_rn(0.f, 0.f);
            uint32_t hin[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
            if (r >= 0) {
                const float4 pw = MODE == 2 && kind == KIND_CACHE ? make_float4(0.f, 0.f, 0.f, 0.f) : p.row_pay[r];
                if (MODE == 2 && kind == KIND_CACHE) {
                    cache_head_input(p.row_lat[r], p.row_out[r].y >> 16, p.latent_offset, hin);
                } else {
                    hash_encode<FVC_TC_HASH_GROUP>(p.grid, p.table, make_float3(pw.x, pw.y, pw.z), feat);
                }
            }
            /* MODE 2: the cache list's tiles skip the density layers (tile is block-uniform) */
            const bool dense = MODE != 2 || tile < res_tiles;
            uint4 b0 = make_uint4(hin[0], hin[1], hin[2], hin[3]), b1 = make_uint4(hin[4], hin[5], hin[6], hin[7]);
            if (dense) {
#pragma unroll
                for (int c = 0; c < 4; ++c) st_chunk(S.X, tid, c, 32, *reinterpret_cast<const uint4 *>(feat + 4 * c));
                if (!(ok = tc_publish(ok))) break;
                /* ---- layer 1: 32 -> 64, ReLU ---- */
                ok = tc_run(S, tmem, S.W + TC_B1, 32, 64, phase);
                epi_hidden(tmem + lane_base, nullptr, S.X, tid);
                if (!(ok = tc_publish(ok))) break;
                /* ---- layer 2: 64 -> 16 (log-density, latents) ---- */
                ok = tc_run(S, tmem, S.W + TC_B2, 64, 16, phase);
                float v[16];
                tmem_ld16(tmem + lane_base, v);
                tmem_wait_ld();
                if (!(MODE == 2 && kind == KIND_CACHE)) {
                    b0 = pack8(v);
                    b1 = pack8(v + 8);
                }
            }
            log_density = (uint16_t)(b0.x & 0xffffu);
            st_chunk(S.X, tid, 0, HK, b0);
            st_chunk(S.X, tid, 1, HK, b1);
        } else {
            /* ---- cache lookup -> head input (log-density, latents) ---- */
            __half hin[32];
            if (r >= 0) {
                cache_row_input(p, k, r, hin);
            } else {
                for (int q = 16; q < 32; ++q) hin[q] = __float2half_rn(0.f);
            }
            log_density = __half_as_ushort(hin[16]);
            st_chunk(S.X, tid, 0, HK, *reinterpret_cast<const uint4 *>(hin + 16));
            st_chunk(S.X, tid, 1, HK, *reinterpret_cast<const uint4 *>(hin + 24));
        }
        st_chunk(S.X, tid, 2, HK, *reinterpret_cast<const uint4 *>(sh));
        st_chunk(S.X, tid, 3, HK, *reinterpret_cast<const uint4 *>(sh + 4));
        if (p.freq) {
            /* the frequency encoding of the row's network input position (include/nerf_network.h:241-246) */
            uint4 fx = make_uint4(0u, 0u, 0u, 0u), fy = fx, fz = fx;
            if (r >= 0) {
                const bool cache_row = MODE == 1 || (MODE == 2 && kind == KIND_CACHE);
                float3 q;
                if (cache_row) {
                    q = cache_row_position(p, states, r);
                } else {
                    const float4 pw = p.row_pay[r];
                    q = make_float3(pw.x, pw.y, pw.z);
                }
                fx = freq_chunk(q.x);
                fy = freq_chunk(q.y);
                fz = freq_chunk(q.z);
            }
            st_chunk(S.X, tid, 4, HK, fx);
            st_chunk(S.X, tid, 5, HK, fy);
            st_chunk(S.X, tid, 6, HK, fz);
            st_chunk(S.X, tid, 7, HK, make_uint4(0u, 0u, 0u, 0u));
        }
        if (!(ok = tc_publish(ok))) break;
        /* ---- head layer 1: (latents | SH (| frequency)) HK -> 64, bias from the 1-padding, ReLU ---- */
        ok = tc_run(S, tmem, S.W + wb3, HK, 64, phase);
        epi_hidden(tmem + lane_base, S.bias3, S.X, tid);
        if (!(ok = tc_publish(ok))) break;
        if (HH == 2) {
            /* ---- head layer 2: 64 -> 64, ReLU ---- */
            ok = tc_run(S, tmem, S.W + wb4, 64, 64, phase);
            epi_hidden(tmem + lane_base, nullptr, S.X, tid);
            if (!(ok = tc_publish(ok))) break;
        }
        /* ---- output layer: 64 -> 16 (rgb logits in cols 0..2) ---- */
        ok = tc_run(S, tmem, S.W + wb5, 64, 16, phase);
        float o[16];
        tmem_ld16(tmem + lane_base, o);
        tmem_wait_ld();
        if (r >= 0)
            p.row_out[r] = make_uint2(pack_h2(o[0], o[1]),
                                      (uint32_t)__half_as_ushort(__float2half_rn(o[2])) | ((uint32_t)log_density << 16));
        tc_fence_before();
        if (__syncthreads_or(!ok)) { ok = false; break; }
    }
    if (!ok && tid == 0) atomicOr(p.guard, 16);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TC_COLS);
    }
}

/* The cache build's density network (NerfNetwork::inferenceLatents on the
 * build rows, src/cache_renderer.cu:1020-1030) on tcgen05: the hash features
 * and the two density layers of wf_net_tc_kernel (same tiles, weights,
 * epilogues and bounded waits), on every row of a build iteration; writes
 * the row's fp16 log-density and its 8 latents from output latent_offset. */
__global__ void __launch_bounds__(128, FVC_TC_CTAS_PER_SM) cache_density_tc_kernel(CacheBuildParams p, const uint8_t *weights_tc,
                                                                                     const int *n_rows_ptr)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
    const int n_rows = *n_rows_ptr;
    if (n_rows == 0) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&S.mbar, 1);
        mbar_arrive_expect_tx(&S.mbar, TC_WBYTES);
        bulk_copy_g2s(S.W, weights_tc, TC_WBYTES, &S.mbar);
    }
    if (warp == 0) tmem_alloc(&S.tmem_base, TC_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    uint32_t phase = 0;
    bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    const int lo = p.latent_offset;
    const int n_tiles = (n_rows + 127) / 128;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int r = tile * 128 + tid;
        __half2 feat[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) feat[q] = __floats2half2_rn(0.f, 0.f);
        if (r < n_rows) {
            const float4 rw = p.build_rows[r];
            hash_encode<FVC_TC_HASH_GROUP>(p.grid, p.table, make_float3(rw.x, rw.y, rw.z), feat);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) st_chunk(S.X, tid, c, 32, *reinterpret_cast<const uint4 *>(feat + 4 * c));
        if (!(ok = tc_publish(ok))) break;
        /* ---- layer 1: 32 -> 64, ReLU ---- */
        ok = tc_run(S, tmem, S.W + TC_B1, 32, 64, phase);
        epi_hidden(tmem + lane_base, nullptr, S.X, tid);
        if (!(ok = tc_publish(ok))) break;
        /* ---- layer 2: 64 -> 16 (log-density, latents) ---- */
        ok = tc_run(S, tmem, S.W + TC_B2, 64, 16, phase);
        float v[16];
        tmem_ld16(tmem + lane_base, v);
        tmem_wait_ld();
        if (r < n_rows) {
            __half h[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) h[j] = __float2half_rn(v[j]);
            p.build_den[r] = h[0];
            uint32_t lw[4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                lw[q] = (uint32_t)__half_as_ushort(h[lo + 2 * q]) | ((uint32_t)__half_as_ushort(h[lo + 2 * q + 1]) << 16);
            p.build_lat[r] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        tc_fence_before();
        if (__syncthreads_or(!ok)) { ok = false; break; }
    }
    if (!ok && tid == 0 && p.guard) atomicOr(p.guard, 16);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TC_COLS);
    }
}

cudaError_t launch_cache_density_tc(const CacheBuildParams &p, const uint8_t *weights_tc, int n_sms, cudaStream_t s)
{
    static PerDeviceOnce once;
    cudaError_t e = once.run([] {
        return cudaFuncSetAttribute(cache_density_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcSmem));
    });
    if (e != cudaSuccess) return e;
    cache_density_tc_kernel<<<n_sms * FVC_TC_CTAS_PER_SM, 128, sizeof(TcSmem), s>>>(p, weights_tc, p.build_row_counter);
    return cudaGetLastError();
}

/* ------------------------------------------------------------------------- */
/* the network on tile heights M = 64 and M = 256 (resample rows)            */
/* ------------------------------------------------------------------------- */
/* The layers, weights, epilogue arithmetic and bounded waits of
 * wf_net_tc_kernel, on other tile heights for the batch autotuner.
 * M = 256: 256 threads, thread t owns row t.  The operand is one 256-row
 * K-major tile and each layer issues two M = 128 MMAs: rows 0..127 into TMEM
 * columns 0..63, rows 128..255 into columns 64..127.  Warp w reads TMEM lanes
 * 32 (w mod 4)..+31 of its half's columns.
 * M = 64: one M = 64 MMA per layer, whose accumulator rows 16q..16q+15 sit in
 * TMEM lanes 32q..32q+15.  128 threads: lanes 0..15 of warp q own rows
 * 16q..16q+15 and run the epilogues; for the hash features both half-warps
 * work on the same 16 rows, lanes 16..31 taking the upper levels, so each
 * thread's chain of dependent gathers is half as long. */
template <int MT>
struct __align__(128) TcmSmem {
    uint8_t W[TC_WBYTES];
    uint8_t X[MT * 64 * 2];
    float bias3[64];
    uint64_t mbar;
    uint32_t tmem_base;
};
template <int MT> __host__ __device__ constexpr int tcm_threads() { return MT == 64 ? 128 : MT; }
template <int MT> __host__ __device__ constexpr int tcm_cols() { return MT == 256 ? 128 : 64; }
template <int MT> __host__ __device__ constexpr int tcm_ctas_per_sm() { return MT == 256 ? 3 : FVC_TC_CTAS_PER_SM; }
static_assert(tcm_ctas_per_sm<256>() * tcm_cols<256>() <= 512 && tcm_ctas_per_sm<64>() * tcm_cols<64>() <= 512,
              "resident CTAs must fit in the SM's 512 TMEM columns");

template <int MT>
__device__ __forceinline__ void tcm_layer(uint32_t tmem, const uint8_t *a, const uint8_t *b, int K, int N)
{
    const uint32_t sbo = (uint32_t)(K / 8) * 128u;
    const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
    const uint32_t id = idesc_f16(MT == 64 ? 64 : 128, N, false);
#pragma unroll
    for (int h = 0; h < (MT == 256 ? 2 : 1); ++h)
        for (int kc = 0; kc < K / 16; ++kc)
            tc_mma_f16(tmem + 64u * h, umma_desc(a0 + (uint32_t)h * 16u * sbo + 256u * kc, 128u, sbo),
                       umma_desc(b0 + 256u * kc, 128u, sbo), id, kc > 0 ? 1u : 0u);
}

template <int MT>
__device__ __forceinline__ bool tcm_run(TcmSmem<MT> &S, uint32_t tmem, const uint8_t *b, int K, int N, uint32_t &phase)
{
    if (threadIdx.x == 0) {
        tc_fence_after();
        tcm_layer<MT>(tmem, S.X, b, K, N);
        tc_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    tc_fence_after();
    return ok;
}

/* epi_hidden with the row's writes limited to the threads that own a row
 * (the TMEM loads are warp-collective and run on every lane) */
__device__ __forceinline__ void epi_hidden_own(uint32_t taddr, const float *bias, uint8_t *dst, int row, bool own)
{
    const __half2 zero = __float2half2_rn(0.0f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float v[32];
        tmem_ld32(taddr + 32 * h, v);
        tmem_wait_ld();
        uint32_t w[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            float2 x = make_float2(v[2 * i], v[2 * i + 1]);
            if (bias) x = __fadd2_rn(x, make_float2(bias[32 * h + 2 * i], bias[32 * h + 2 * i + 1]));
            const __half2 r = __hmax2(__float22half2_rn(x), zero);
            w[i] = *reinterpret_cast<const uint32_t *>(&r);
        }
        if (own) {
#pragma unroll
            for (int q = 0; q < 4; ++q) st_chunk(dst, row, 4 * h + q, 64, make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]));
        }
    }
}

template <int MT, int HH, bool LIST>
__global__ void __launch_bounds__(tcm_threads<MT>(), tcm_ctas_per_sm<MT>()) wf_net_tcm_kernel(RenderParams p, int it)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcmSmem<MT> &S = *reinterpret_cast<TcmSmem<MT> *>(smem_raw);
    const int n_rows = LIST ? p.counters[3] : p.counters[2];
    if (n_rows == 0) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int trow = MT == 64 ? 16 * warp + (lane & 15) : tid; /* the tile row this thread works on */
    const bool own = MT == 64 ? lane < 16 : true;                /* ... and whose epilogues it runs */
    const int upper = MT == 64 ? lane >> 4 : 0;
    if (tid == 0) {
        mbar_init(&S.mbar, 1);
        mbar_arrive_expect_tx(&S.mbar, TC_WBYTES);
        bulk_copy_g2s(S.W, p.weights_tc, TC_WBYTES, &S.mbar);
    }
    if (tid < 64) S.bias3[tid] = p.bias3[tid];
    if (warp == 0) tmem_alloc(&S.tmem_base, tcm_cols<MT>());
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (MT == 256 && tid >= 128 ? 64u : 0u);
    const RayState *states = p.states[it & 1];
    /* levels of the lower half-warp (M = 64): a multiple of 4, so each half writes whole 8-value chunks
     * (chunk c holds features 8c..8c+7: levels 4c..4c+3 of 2 features, 2c..2c+1 of 4) */
    const int l_split = 4 * ((p.grid.n_levels + 7) / 8);
    const int c_split = l_split * p.grid.F / 8;
    uint32_t phase = 0;
    bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    const int n_tiles = (n_rows + MT - 1) / MT;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int k = tile * MT + trow;
        const int r = k < n_rows ? (LIST ? p.res_list[k] : k) : -1;
        /* ---- hash features -> tile (K = 32) ---- */
        __half2 feat[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) feat[q] = __floats2half2_rn(0.f, 0.f);
        const int lb = upper ? l_split : 0, le = upper ? p.grid.n_levels : min(l_split, p.grid.n_levels);
        if (r >= 0) {
            const float4 pw = p.row_pay[r];
            if (MT == 64) hash_encode_levels<FVC_TC_HASH_GROUP>(p.grid, p.table, make_float3(pw.x, pw.y, pw.z), feat, lb, le);
            else hash_encode<FVC_TC_HASH_GROUP>(p.grid, p.table, make_float3(pw.x, pw.y, pw.z), feat);
        }
        if (MT == 64) {
            const int c0 = upper ? c_split : 0, c1 = upper ? 4 : c_split;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (c >= c0 && c < c1) st_chunk(S.X, trow, c, 32, *reinterpret_cast<const uint4 *>(feat + 4 * c));
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) st_chunk(S.X, trow, c, 32, *reinterpret_cast<const uint4 *>(feat + 4 * c));
        }
        if (!(ok = tc_publish(ok))) break;
        /* ---- layer 1: 32 -> 64, ReLU ---- */
        ok = tcm_run<MT>(S, tmem, S.W + TC_B1, 32, 64, phase);
        epi_hidden_own(taddr, nullptr, S.X, trow, own);
        if (!(ok = tc_publish(ok))) break;
        /* ---- layer 2: 64 -> 16 (log-density, latents) ---- */
        ok = tcm_run<MT>(S, tmem, S.W + TC_B2, 64, 16, phase);
        uint16_t log_density = 0;
        {
            float v[16];
            tmem_ld16(taddr, v);
            tmem_wait_ld();
            const uint4 b0 = pack8(v), b1 = pack8(v + 8);
            log_density = (uint16_t)(b0.x & 0xffffu);
            __half2 sh[8];
            if (r >= 0 && own) sh16(dir01_of(states, p.row_slot[r]), sh);
            else for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
            if (own) {
                st_chunk(S.X, trow, 0, 32, b0);
                st_chunk(S.X, trow, 1, 32, b1);
                st_chunk(S.X, trow, 2, 32, *reinterpret_cast<const uint4 *>(sh));
                st_chunk(S.X, trow, 3, 32, *reinterpret_cast<const uint4 *>(sh + 4));
            }
        }
        if (!(ok = tc_publish(ok))) break;
        /* ---- head layer 1: (latents | SH) 32 -> 64, bias from the 1-padding, ReLU ---- */
        ok = tcm_run<MT>(S, tmem, S.W + TC_B3, 32, 64, phase);
        epi_hidden_own(taddr, S.bias3, S.X, trow, own);
        if (!(ok = tc_publish(ok))) break;
        if (HH == 2) {
            /* ---- head layer 2: 64 -> 64, ReLU ---- */
            ok = tcm_run<MT>(S, tmem, S.W + TC_B4, 64, 64, phase);
            epi_hidden_own(taddr, nullptr, S.X, trow, own);
            if (!(ok = tc_publish(ok))) break;
        }
        /* ---- output layer: 64 -> 16 (rgb logits in cols 0..2) ---- */
        ok = tcm_run<MT>(S, tmem, S.W + TC_B5, 64, 16, phase);
        float o[16];
        tmem_ld16(taddr, o);
        tmem_wait_ld();
        if (r >= 0 && own)
            p.row_out[r] = make_uint2(pack_h2(o[0], o[1]),
                                      (uint32_t)__half_as_ushort(__float2half_rn(o[2])) | ((uint32_t)log_density << 16));
        tc_fence_before();
        if (__syncthreads_or(!ok)) { ok = false; break; }
    }
    if (!ok && tid == 0) atomicOr(p.guard, 16);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, tcm_cols<MT>());
    }
}

/* ------------------------------------------------------------------------- */
/* tcgen05 network kernel at reduced precision (plain path, resample rows)   */
/* ------------------------------------------------------------------------- */
/* PREC 1, BF16: kind::f16 with bf16 operands; hash features, SH and every
 * layer output are rounded to bf16.
 * PREC 2, FP8-E4M3: kind::f8f6f4 (K = 32 per MMA, the same 8-row x 16-byte
 * core matrices).  Each weight matrix is stored scaled by 448 / amax(W) (per
 * layer, on the host); each activation row is scaled by 448 / amax(row) before
 * its e4m3 conversion.  The thread that owns a row divides both scales out of
 * its fp32 accumulator row in the epilogue.
 * Layer structure, TMEM use, waits and the guard are those of
 * wf_net_tc_kernel; compositing stays fp32. */
__device__ __forceinline__ uint32_t pack_bf2(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ uint32_t pack_e4m3x4(float a, float b, float c, float d)
{
    const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(a, b), __NV_SATFINITE, __NV_E4M3);
    const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(c, d), __NV_SATFINITE, __NV_E4M3);
    return lo | (hi << 16);
}

/* writes this thread's row of K values into the operand tile in the kernel's
 * precision; returns the factor that undoes the row's scale (1 for bf16) */
template <int PREC, int K>
__device__ __forceinline__ float put_row(uint8_t *tile, int row, const float *v)
{
    if (PREC == 1) {
#pragma unroll
        for (int c = 0; c < K / 8; ++c)
            *reinterpret_cast<uint4 *>(tile + kmajor_offset(row, 8 * c, K)) =
                make_uint4(pack_bf2(v[8 * c], v[8 * c + 1]), pack_bf2(v[8 * c + 2], v[8 * c + 3]),
                           pack_bf2(v[8 * c + 4], v[8 * c + 5]), pack_bf2(v[8 * c + 6], v[8 * c + 7]));
        return 1.0f;
    } else {
        float amax = 0.0f;
#pragma unroll
        for (int i = 0; i < K; ++i) amax = fmaxf(amax, fabsf(v[i]));
        const float sc = amax > 0.0f ? 448.0f / amax : 1.0f;
#pragma unroll
        for (int c = 0; c < K / 16; ++c) {
            const float *w = v + 16 * c;
            *reinterpret_cast<uint4 *>(tile + kmajor_offset8(row, 16 * c, K)) =
                make_uint4(pack_e4m3x4(w[0] * sc, w[1] * sc, w[2] * sc, w[3] * sc),
                           pack_e4m3x4(w[4] * sc, w[5] * sc, w[6] * sc, w[7] * sc),
                           pack_e4m3x4(w[8] * sc, w[9] * sc, w[10] * sc, w[11] * sc),
                           pack_e4m3x4(w[12] * sc, w[13] * sc, w[14] * sc, w[15] * sc));
        }
        return 1.0f / sc;
    }
}

template <int PREC>
__device__ __forceinline__ bool tc_run_prec(TcSmem &S, uint32_t tmem, const uint8_t *b, int K, int N, uint32_t &phase)
{
    if (threadIdx.x == 0) {
        tc_fence_after();
        const uint32_t a0 = smem_u32(S.X), b0 = smem_u32(b);
        if (PREC == 1) {
            const uint32_t sbo = (uint32_t)(K / 8) * 128u, id = idesc_f16(128, N, true);
            for (int kc = 0; kc < K / 16; ++kc)
                tc_mma_f16(tmem, umma_desc(a0 + 256u * kc, 128u, sbo), umma_desc(b0 + 256u * kc, 128u, sbo), id, kc > 0 ? 1u : 0u);
        } else {
            const uint32_t sbo = (uint32_t)(K / 16) * 128u, id = idesc_f8_e4m3(128, N);
            for (int kc = 0; kc < K / 32; ++kc)
                tc_mma_f8(tmem, umma_desc(a0 + 256u * kc, 128u, sbo), umma_desc(b0 + 256u * kc, 128u, sbo), id, kc > 0 ? 1u : 0u);
        }
        tc_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    tc_fence_after();
    return ok;
}

/* 64 accumulator columns -> scale, (+bias), ReLU -> next operand row */
template <int PREC>
__device__ __forceinline__ float epi_hidden_prec(uint32_t taddr, float deq, const float *bias, uint8_t *dst, int row)
{
    float v[64];
    tmem_ld32(taddr, *reinterpret_cast<float(*)[32]>(v));
    tmem_ld32(taddr + 32, *reinterpret_cast<float(*)[32]>(v + 32));
    tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i] * deq + (bias ? bias[i] : 0.0f), 0.0f);
    return put_row<PREC, 64>(dst, row, v);
}

constexpr int TC_PREC_CTAS_PER_SM = 4; /* 128 registers: the fp32 rows of the scaled epilogues */

template <int PREC, int HH>
__global__ void __launch_bounds__(128, TC_PREC_CTAS_PER_SM) wf_net_tc_prec_kernel(RenderParams p, int it)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
    const int n_rows = p.counters[2];
    if (n_rows == 0) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint8_t *wsrc = PREC == 1 ? p.weights_tc_bf16 : p.weights_tc_fp8;
    const int wbytes = PREC == 1 ? TC_WBYTES : TC8_WBYTES;
    if (tid == 0) { /* the weights by one bulk copy, completing phase 0 (as wf_net_tc_kernel) */
        mbar_init(&S.mbar, 1);
        mbar_arrive_expect_tx(&S.mbar, (uint32_t)wbytes);
        bulk_copy_g2s(S.W, wsrc, (uint32_t)wbytes, &S.mbar);
    }
    if (tid < 64) S.bias3[tid] = p.bias3[tid];
    if (warp == 0) tmem_alloc(&S.tmem_base, TC_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    float iw[5] = {1.f, 1.f, 1.f, 1.f, 1.f};
    if (PREC == 2)
#pragma unroll
        for (int l = 0; l < 5; ++l) iw[l] = __ldg(p.tc_fp8_iw + l);
    const int o1 = PREC == 1 ? TC_B1 : TC8_B1, o2 = PREC == 1 ? TC_B2 : TC8_B2, o3 = PREC == 1 ? TC_B3 : TC8_B3,
              o4 = PREC == 1 ? TC_B4 : TC8_B4, o5 = PREC == 1 ? TC_B5 : TC8_B5;
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const RayState *states = p.states[it & 1];
    uint32_t phase = 0;
    bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    const int n_tiles = (n_rows + 127) / 128;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int r = tile * 128 + tid < n_rows ? tile * 128 + tid : -1;
        float in[32];
        __half2 feat[16];
        float3 d01 = make_float3(0.5f, 0.5f, 0.5f);
        if (r >= 0) {
            const float4 pw = p.row_pay[r];
            hash_encode<FVC_TC_HASH_GROUP>(p.grid, p.table, make_float3(pw.x, pw.y, pw.z), feat);
            d01 = dir01_of(states, p.row_slot[r]);
        } else {
#pragma unroll
            for (int q = 0; q < 16; ++q) feat[q] = __floats2half2_rn(0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const float2 f = __half22float2(feat[q]);
            in[2 * q] = f.x;
            in[2 * q + 1] = f.y;
        }
        float deq = put_row<PREC, 32>(S.X, tid, in);
        if (!(ok = tc_publish(ok))) break;
        /* density network */
        ok = tc_run_prec<PREC>(S, tmem, S.W + o1, 32, 64, phase);
        deq = epi_hidden_prec<PREC>(tmem + lane_base, deq * iw[0], nullptr, S.X, tid);
        if (!(ok = tc_publish(ok))) break;
        ok = tc_run_prec<PREC>(S, tmem, S.W + o2, 64, 16, phase);
        float o[16];
        tmem_ld16(tmem + lane_base, o);
        tmem_wait_ld();
        const float dq2 = deq * iw[1];
        const float log_density = o[0] * dq2;
        /* head input [layer-2 outputs (latents only) | SH] in the remapped order of W3 */
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int lat = j - p.latent_offset;
            const float v = o[j] * dq2;
            in[j] = (lat >= 0 && lat < 8) ? (PREC == 1 ? __bfloat162float(__float2bfloat16_rn(v)) : v) : 0.0f;
        }
        {
            __half2 sh[8];
            sh16(d01, sh);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float2 f = __half22float2(sh[q]);
                in[16 + 2 * q] = f.x;
                in[17 + 2 * q] = f.y;
            }
        }
        deq = put_row<PREC, 32>(S.X, tid, in);
        if (!(ok = tc_publish(ok))) break;
        /* color head */
        ok = tc_run_prec<PREC>(S, tmem, S.W + o3, 32, 64, phase);
        deq = epi_hidden_prec<PREC>(tmem + lane_base, deq * iw[2], S.bias3, S.X, tid);
        if (!(ok = tc_publish(ok))) break;
        if (HH == 2) {
            ok = tc_run_prec<PREC>(S, tmem, S.W + o4, 64, 64, phase);
            deq = epi_hidden_prec<PREC>(tmem + lane_base, deq * iw[3], nullptr, S.X, tid);
            if (!(ok = tc_publish(ok))) break;
        }
        ok = tc_run_prec<PREC>(S, tmem, S.W + o5, 64, 16, phase);
        tmem_ld16(tmem + lane_base, o);
        tmem_wait_ld();
        const float dq5 = deq * iw[4];
        /* outputs in the network's precision, stored as fp16 like the fp16 path */
        auto rnd = [](float v) { return PREC == 1 ? __bfloat162float(__float2bfloat16_rn(v)) : v; };
        if (r >= 0)
            p.row_out[r] = make_uint2(pack_h2(rnd(o[0] * dq5), rnd(o[1] * dq5)),
                                      (uint32_t)__half_as_ushort(__float2half_rn(rnd(o[2] * dq5))) |
                                          ((uint32_t)__half_as_ushort(__float2half_rn(rnd(log_density))) << 16));
        tc_fence_before();
        if (__syncthreads_or(!ok)) { ok = false; break; }
    }
    if (!ok && tid == 0) atomicOr(p.guard, 16);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TC_COLS);
    }
}

/* ------------------------------------------------------------------------- */
/* composite + compaction                                                    */
/* ------------------------------------------------------------------------- */
template <bool CACHED>
__global__ void __launch_bounds__(128) wf_composite_kernel(RenderParams p, int it)
{
    const int n_alive = p.counters[it & 1];
    RayState *cur = p.states[it & 1], *nxt = p.states[(it + 1) & 1];
    for (int base = blockIdx.x * blockDim.x; base < n_alive; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool valid = i < n_alive;
        bool keep = false;
        RayState st;
        int n_comp = 0;
        unsigned long long why = 0; /* rows per REASON_* 1..7, 8 bits each (at most S_ROWS rows a ray and sub-iteration) */
        if (valid) {
            st = cur[i];
            const int2 rr = p.ray_rows[i];
            float4 acc = st.acc, comp = st.comp;
            int c_res = st.cnt.y, c_cache = st.cnt.z, c_drop = st.cnt2.x;
            float w_res = 0.f, w_cache = 0.f; /* this sub-iteration's contribution weights (DEBUG form, :867-871) */
            bool term = false;
            /* rows are in t order: the merge of the resample and cache
             * streams of accumulate_cache_perf_kernel (:270-304) */
            for (int j = 0; j < rr.y; ++j) {
                const int r = rr.x + j;
                const int code = CACHED ? (int)p.row_kind[r] : KIND_RESAMPLE;
                const int kind = row_kind_of(code);
                if (CACHED && kind != KIND_SKIP && row_reason_of(code)) why += 1ull << ((8 * (row_reason_of(code) - 1)) & 63);
                if (kind >= KIND_DROP) {
                    c_drop += kind == KIND_DROP;
                    continue;
                }
                if (kind == KIND_CACHE) ++c_cache; else ++c_res;
                ++n_comp;
                const uint2 ov = p.row_out[r];
                const float t0 = p.row_t0[r];
                const float2 rg = __half22float2(*reinterpret_cast<const __half2 *>(&ov.x));
                const float lb = __half2float(__ushort_as_half((unsigned short)(ov.y & 0xffffu)));
                const float ld = __half2float(__ushort_as_half((unsigned short)(ov.y >> 16)));
                const float dt = calc_step(p.steps, t0);
                /* the basic cache renderer composites a cache row with its looked-up density
                 * (accumulate_cache_render_kernel, src/cache_basic_renderer.cu:255-258) */
                const float sigma = CACHED && p.basic_cache && kind == KIND_CACHE ? p.row_pay[r].w : expf(ld);
                const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-sigma * dt)));
                if (alpha > p.scene.alpha_thre) {
                    const float wgt = alpha * acc.w;
                    kahan_add(acc.x, comp.x, wgt / (1.0f + expf(-rg.x)));
                    kahan_add(acc.y, comp.y, wgt / (1.0f + expf(-rg.y)));
                    kahan_add(acc.z, comp.z, wgt / (1.0f + expf(-lb)));
                    acc.w *= 1.0f - alpha;
                    if (CACHED) {
                        if (kind == KIND_CACHE) w_cache += wgt;
                        else w_res += wgt;
                    }
                }
                if (acc.w < 1e-4f) { term = true; break; }
            }
            if (CACHED) { /* one ray a pixel: no other thread adds to it in this launch */
                if (p.contrib_res) p.contrib_res[st.cnt.x] += w_res;
                if (p.contrib_cache) p.contrib_cache[st.cnt.x] += w_cache;
            }
            st.acc = acc;
            st.comp = comp;
            st.cnt.y = c_res;
            st.cnt.z = c_cache;
            st.cnt2.x = c_drop;
            if (term || st.cnt2.y) {
                write_pixel(p, st.cnt.x, acc, make_int4(c_res, c_cache, c_drop, st.cnt.w));
            } else {
                keep = true;
            }
        }
        const int ws = __reduce_add_sync(FULLMASK, n_comp);
        if (lane_id() == 0 && ws) atomicAdd(&p.stats->n_samples, (unsigned long long)ws);
        if (CACHED && __any_sync(FULLMASK, why != 0)) {
#pragma unroll
            for (int q = 1; q < N_REASONS; ++q) {
                const unsigned c = __reduce_add_sync(FULLMASK, (unsigned)(why >> (8 * (q - 1))) & 255u);
                if (lane_id() == 0 && c) atomicAdd(&p.stats->n_reason[q], (unsigned long long)c);
            }
        }
        const unsigned m = __ballot_sync(FULLMASK, keep);
        int nb = 0;
        if (lane_id() == 0 && m) nb = atomicAdd(p.counters + ((it + 1) & 1), __popc(m));
        nb = __shfl_sync(FULLMASK, nb, 0);
        if (keep) nxt[nb + __popc(m & lane_lt())] = st;
    }
}

/* Adjoint of front-to-back compositing for this sub-iteration's rows (plain
 * path).  Per ray, in sample order, with g = dL/dC and X_total from the loss
 * kernel, X_prefix in acc.x and T in acc.w of the ray state:
 *   X_prefix += T alpha g.c;  T' = T (1 - alpha);
 *   dL/dsigma = dt (T' g.c - (X_total - X_prefix));  dL/dc = T alpha g.
 * The alpha threshold and the T < 1e-4 termination follow the forward
 * compositing exactly, so the rows that composited get gradients and no
 * other; rows the forward skipped (known-empty cache voxels) get none.  Rows
 * with a gradient are listed per stream: grad_res_list (counters[6]),
 * grad_cache_list (counters[7]). */
template <bool CACHED>
__global__ void __launch_bounds__(128) wf_composite_bwd_kernel(RenderParams p, int it)
{
    const int n_alive = p.counters[it & 1];
    RayState *cur = p.states[it & 1], *nxt = p.states[(it + 1) & 1];
    for (int base = blockIdx.x * blockDim.x; base < n_alive; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool valid = i < n_alive;
        bool keep = false;
        RayState st;
        int n_res = 0, n_cch = 0;
        int2 rr = make_int2(0, 0);
        uint32_t gmask = 0, cmask = 0;
        if (valid) {
            st = cur[i];
            rr = p.ray_rows[i];
            const float4 rg = p.ray_grad[st.cnt.x];
            float T = st.acc.w, xp = st.acc.x;
            bool term = false;
            for (int j = 0; j < rr.y; ++j) {
                const int r = rr.x + j;
                float4 dout = make_float4(0.f, 0.f, 0.f, 0.f);
                const int kind = CACHED ? row_kind_of(p.row_kind[r]) : KIND_RESAMPLE;
                if (!term && kind < KIND_DROP) {
                    const uint2 ov = p.row_out[r];
                    const float t0 = p.row_t0[r];
                    const float2 lg = __half22float2(*reinterpret_cast<const __half2 *>(&ov.x));
                    const float lb = __half2float(__ushort_as_half((unsigned short)(ov.y & 0xffffu)));
                    const float ld = __half2float(__ushort_as_half((unsigned short)(ov.y >> 16)));
                    const float dt = calc_step(p.steps, t0);
                    const float sigma = expf(ld);
                    const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-sigma * dt)));
                    if (alpha > p.scene.alpha_thre) {
                        const float c0 = 1.0f / (1.0f + expf(-lg.x)), c1 = 1.0f / (1.0f + expf(-lg.y)),
                                    c2 = 1.0f / (1.0f + expf(-lb));
                        const float gc = rg.x * c0 + rg.y * c1 + rg.z * c2;
                        const float ta = T * alpha;
                        xp += ta * gc;
                        const float Tn = T * (1.0f - alpha);
                        const float dsig = dt * (Tn * gc - (rg.w - xp));
                        dout = make_float4(rg.x * ta * c0 * (1.0f - c0), rg.y * ta * c1 * (1.0f - c1), rg.z * ta * c2 * (1.0f - c2),
                                           dsig * sigma);
                        T = Tn;
                        if (kind == KIND_CACHE) { cmask |= 1u << j; ++n_cch; }
                        else { gmask |= 1u << j; ++n_res; }
                    }
                    if (T < 1e-4f) term = true;
                }
                p.row_dout[r] = dout;
            }
            st.acc.x = xp;
            st.acc.w = T;
            keep = !(term || st.cnt2.y);
        }
        /* list the rows with a gradient per network stream (one atomic per warp and list) */
        auto append = [&](int n, uint32_t mask, int *list, int *counter) {
            int incl = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULLMASK, incl, o);
                if (lane_id() >= o) incl += v;
            }
            const int total = __shfl_sync(FULLMASK, incl, 31);
            int lb = 0;
            if (lane_id() == 0 && total) lb = atomicAdd(counter, total);
            lb = __shfl_sync(FULLMASK, lb, 0) + incl - n;
            for (uint32_t mm = mask; mm; mm &= mm - 1) list[lb++] = rr.x + __ffs(mm) - 1;
        };
        append(n_res, gmask, p.grad_res_list, p.counters + 6);
        if (CACHED) append(n_cch, cmask, p.grad_cache_list, p.counters + 7);
        const unsigned m = __ballot_sync(FULLMASK, keep);
        int nb = 0;
        if (lane_id() == 0 && m) nb = atomicAdd(p.counters + ((it + 1) & 1), __popc(m));
        nb = __shfl_sync(FULLMASK, nb, 0);
        if (keep) nxt[nb + __popc(m & lane_lt())] = st;
    }
}

/* resets the row counters after the kernels of the sub-iteration consumed them */
__global__ void wf_reset_rows_kernel(RenderParams p, int cached)
{
    if (threadIdx.x == 0) {
        atomicAdd(&p.stats->n_resamples, (unsigned long long)(cached ? p.counters[3] : p.counters[2]));
        atomicAdd(&p.stats->n_cache_hits, (unsigned long long)p.counters[4]);
        atomicAdd(&p.stats->n_dropped, (unsigned long long)(cached ? p.counters[2] - p.counters[3] - p.counters[4] : 0));
        p.counters[2] = 0;
        p.counters[3] = 0;
        p.counters[4] = 0;
        p.counters[6] = 0;
        p.counters[7] = 0;
    }
}

/* ------------------------------------------------------------------------- */
/* host side                                                                 */
/* ------------------------------------------------------------------------- */
/* ------------------------------------------------------------------------- */
/* the view-dependent split network on tcgen05                               */
/* ------------------------------------------------------------------------- */
/* NerfNetwork::init_viewdep / inferenceLatents / inferenceHead
 * (include/nerf_network.h:120-158,173-266) for models with mlp_first_head.
 * The layer structure, TMEM use (64 columns), waits and guard are those of
 * wf_net_tc_kernel, with:
 *   - resample rows (MODE 0): after the density network, the first head on
 *     [density outputs 16 | SH of the initial direction 16] (32 -> 64 -> 16);
 *     its outputs take the head-input rows 1..16, row 0 keeps the
 *     log-density.  The initial direction of a resample row is its own, so
 *     the SH difference is zero (the reference clears that buffer when both
 *     inputs are the same matrix);
 *   - cache rows (MODE 1): the looked-up latents, and the SH difference
 *     between the ray direction and the cache camera's direction to the
 *     sample (written by the classification into the row payload), rounded
 *     to fp16 and subtracted in fp16 as the reference's sub kernel;
 *   - the color head's input [latents 8 | SH 16 | SH difference 16 |
 *     1-padding 8] as one K = 48 tile; the padding columns of its weights
 *     give the bias.
 * 45 KB of shared memory: four CTAs per SM. */
struct __align__(128) VdSmem {
    uint8_t W[VDF_WBYTES]; /* VD_WBYTES unless the head has the frequency encoding */
    uint8_t X[128 * 64 * 2];
    uint64_t mbar;
    uint32_t tmem_base;
};

__device__ __forceinline__ bool vd_run(VdSmem &S, uint32_t tmem, const uint8_t *b, int K, int N, uint32_t &phase)
{
    if (threadIdx.x == 0) {
        tc_fence_after();
        tc_layer(tmem, S.X, b, K, N);
        tc_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    tc_fence_after();
    return ok;
}

template <int MODE, int HH, bool LIST>
__global__ void __launch_bounds__(128, 4) wf_net_vd_kernel(RenderParams p, int it)
{
    extern __shared__ __align__(128) unsigned char vd_smem_raw[];
    VdSmem &S = *reinterpret_cast<VdSmem *>(vd_smem_raw);
    const int n_rows = MODE == 0 ? (LIST ? p.counters[3] : p.counters[2]) : p.counters[4];
    if (n_rows == 0) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    /* the color head's input: K = 48 with the 1-padding, or K = 64 with the frequency encoding */
    const int HK = p.freq ? 64 : 48;
    const int wb4 = p.freq ? VDF_B4 : VD_B4, wb5 = p.freq ? VDF_B5 : VD_B5;
    if (tid == 0) {
        const int wbytes = p.freq ? VDF_WBYTES : VD_WBYTES;
        mbar_init(&S.mbar, 1);
        mbar_arrive_expect_tx(&S.mbar, wbytes);
        bulk_copy_g2s(S.W, p.weights_vd, wbytes, &S.mbar);
    }
    if (warp == 0) tmem_alloc(&S.tmem_base, TC_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const RayState *states = p.states[it & 1];
    const int lo = p.latent_offset;
    uint32_t phase = 0;
    bool ok = mbar_wait(&S.mbar, phase, TC_WAIT_LIMIT);
    phase ^= 1u;
    const int n_tiles = (n_rows + 127) / 128;
    const uint32_t one2 = pack_h2(1.0f, 1.0f);
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int k = tile * 128 + tid;
        const int r = k < n_rows ? (MODE == 0 ? (LIST ? p.res_list[k] : k) : p.cache_list[k]) : -1;
        __half2 sh[8];
        if (r >= 0) sh16(dir01_of(states, p.row_slot[r]), sh);
        else for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
        uint16_t log_density = 0;
        uint4 lat = make_uint4(0u, 0u, 0u, 0u), diff0 = make_uint4(0u, 0u, 0u, 0u), diff1 = make_uint4(0u, 0u, 0u, 0u);
        if (MODE == 0) {
            /* ---- hash features -> tile (K = 32) ---- */
            __half2 feat[16];
            if (r >= 0) {
                const float4 pw = p.row_pay[r];
                hash_encode<FVC_TC_HASH_GROUP>(p.grid, p.table, make_float3(pw.x, pw.y, pw.z), feat);
            } else {
                for (int q = 0; q < 16; ++q) feat[q] = __floats2half2_rn(0.f, 0.f);
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) st_chunk(S.X, tid, c, 32, *reinterpret_cast<const uint4 *>(feat + 4 * c));
            if (!(ok = tc_publish(ok))) break;
            ok = vd_run(S, tmem, S.W + VD_B1, 32, 64, phase);
            epi_hidden(tmem + lane_base, nullptr, S.X, tid);
            if (!(ok = tc_publish(ok))) break;
            /* ---- density outputs (16, fp16) ---- */
            ok = vd_run(S, tmem, S.W + VD_B2, 64, 16, phase);
            float v[16];
            tmem_ld16(tmem + lane_base, v);
            tmem_wait_ld();
            const uint4 b0 = pack8(v), b1 = pack8(v + 8);
            log_density = (uint16_t)(b0.x & 0xffffu);
            /* ---- first head on [density outputs | SH of the initial direction] ---- */
            st_chunk(S.X, tid, 0, 32, b0);
            st_chunk(S.X, tid, 1, 32, b1);
            st_chunk(S.X, tid, 2, 32, *reinterpret_cast<const uint4 *>(sh));
            st_chunk(S.X, tid, 3, 32, *reinterpret_cast<const uint4 *>(sh + 4));
            if (!(ok = tc_publish(ok))) break;
            ok = vd_run(S, tmem, S.W + VD_F1, 32, 64, phase);
            epi_hidden(tmem + lane_base, nullptr, S.X, tid);
            if (!(ok = tc_publish(ok))) break;
            ok = vd_run(S, tmem, S.W + VD_F2, 64, 16, phase);
            float f[16];
            tmem_ld16(tmem + lane_base, f);
            tmem_wait_ld();
            /* head-input rows lo .. lo + 7: row 0 the log-density, rows 1.. the first head's outputs */
            float lv[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) lv[j] = lo ? f[j] : (j == 0 ? __half2float(__ushort_as_half(log_density)) : f[j - 1]);
            lat = pack8(lv);
        } else {
            /* ---- looked-up latents and the SH difference to the cache camera's direction ---- */
            if (r >= 0) {
                lat = p.row_lat[k];
                const uint32_t ld = p.row_out[r].y >> 16;
                log_density = (uint16_t)(lo == 0 ? (lat.x & 0xffffu) : ld);
                const float4 iv = p.row_pay[r];
                __half2 shi[8], df[8];
                sh16(make_float3(iv.x, iv.y, iv.z), shi);
#pragma unroll
                for (int q = 0; q < 8; ++q) df[q] = __hsub2(sh[q], shi[q]);
                diff0 = *reinterpret_cast<const uint4 *>(df);
                diff1 = *reinterpret_cast<const uint4 *>(df + 4);
            }
        }
        /* ---- color head input [latents | SH | SH difference | 1-padding or frequency encoding] ---- */
        st_chunk(S.X, tid, 0, HK, lat);
        st_chunk(S.X, tid, 1, HK, *reinterpret_cast<const uint4 *>(sh));
        st_chunk(S.X, tid, 2, HK, *reinterpret_cast<const uint4 *>(sh + 4));
        st_chunk(S.X, tid, 3, HK, diff0);
        st_chunk(S.X, tid, 4, HK, diff1);
        if (p.freq) {
            /* the frequency encoding of the row's network input position (include/nerf_network.h:55-81,
             * src/my_fully_fused_mlp.cu:20-100) */
            uint4 fx = make_uint4(0u, 0u, 0u, 0u), fy = fx, fz = fx;
            if (r >= 0) {
                float3 q;
                if (MODE == 1) {
                    q = cache_row_position(p, states, r);
                } else {
                    const float4 pw = p.row_pay[r];
                    q = make_float3(pw.x, pw.y, pw.z);
                }
                fx = freq_chunk(q.x);
                fy = freq_chunk(q.y);
                fz = freq_chunk(q.z);
            }
            st_chunk(S.X, tid, 5, HK, fx);
            st_chunk(S.X, tid, 6, HK, fy);
            st_chunk(S.X, tid, 7, HK, fz);
        } else {
            st_chunk(S.X, tid, 5, HK, make_uint4(one2, one2, one2, one2));
        }
        if (!(ok = tc_publish(ok))) break;
        ok = vd_run(S, tmem, S.W + VD_B3, HK, 64, phase);
        epi_hidden(tmem + lane_base, nullptr, S.X, tid);
        if (!(ok = tc_publish(ok))) break;
        if (HH == 2) {
            ok = vd_run(S, tmem, S.W + wb4, 64, 64, phase);
            epi_hidden(tmem + lane_base, nullptr, S.X, tid);
            if (!(ok = tc_publish(ok))) break;
        }
        ok = vd_run(S, tmem, S.W + wb5, 64, 16, phase);
        float o[16];
        tmem_ld16(tmem + lane_base, o);
        tmem_wait_ld();
        if (r >= 0)
            p.row_out[r] = make_uint2(pack_h2(o[0], o[1]),
                                      (uint32_t)__half_as_ushort(__float2half_rn(o[2])) | ((uint32_t)log_density << 16));
        tc_fence_before();
        if (__syncthreads_or(!ok)) { ok = false; break; }
    }
    if (!ok && tid == 0) atomicOr(p.guard, 16);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TC_COLS);
    }
}

template <int HH>
static cudaError_t set_net_attrs()
{
    const int smem = (int)sizeof(NetSmem);
    cudaError_t e = cudaFuncSetAttribute(wf_net_resample_kernel<HH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_resample_kernel<HH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_cache_kernel<HH>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    const int tsmem = (int)tc_smem_bytes(1); /* the largest launch (a head with the frequency encoding) */
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tc_kernel<0, HH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tc_kernel<0, HH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tc_kernel<1, HH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tc_kernel<2, HH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tcm_kernel<64, HH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcmSmem<64>));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tcm_kernel<256, HH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcmSmem<256>));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tc_prec_kernel<1, HH>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_tc_prec_kernel<2, HH>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
    const int vsmem = (int)sizeof(VdSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_vd_kernel<0, HH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, vsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_vd_kernel<0, HH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, vsmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_vd_kernel<1, HH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, vsmem);
    return e;
}

template <int HH>
static cudaError_t ensure_net_attrs()
{
    static PerDeviceOnce once;
    return once.run([] { return set_net_attrs<HH>(); });
}

/* The cached render's sub-iteration as march-with-classification + one network launch over all rows
 * (wf_net_tc_kernel MODE 2): the performance cache renderer on the tcgen05 path with the density head.
 * The basic cache renderer, view-dependent heads and the mma.sync path keep the classification kernel
 * and the two row lists. */
static inline bool fused_cached_path(const RenderParams &p)
{
    return p.fused_classify && !p.basic_cache && !p.view_dependent && p.use_tc;
}

/* the network kernel of the plain path's rows in the renderer's network path and precision */
template <int HH>
static void launch_plain_net(const RenderParams &p, int it, int n_sms, cudaStream_t s)
{
    const size_t tc_smem = tc_smem_bytes(p.freq);
    const int grid_tc = n_sms * FVC_TC_CTAS_PER_SM;
    if (p.view_dependent) wf_net_vd_kernel<0, HH, false><<<n_sms * 4, 128, sizeof(VdSmem), s>>>(p, it);
    else if (!p.use_tc) wf_net_resample_kernel<HH, false><<<n_sms * 2, NET_WARPS * 32, sizeof(NetSmem), s>>>(p, it);
    else if (p.precision == 1) wf_net_tc_prec_kernel<1, HH><<<n_sms * TC_PREC_CTAS_PER_SM, 128, tc_smem, s>>>(p, it);
    else if (p.precision == 2) wf_net_tc_prec_kernel<2, HH><<<n_sms * TC_PREC_CTAS_PER_SM, 128, tc_smem, s>>>(p, it);
    else if (p.m_tile == 64)
        wf_net_tcm_kernel<64, HH, false><<<n_sms * tcm_ctas_per_sm<64>(), tcm_threads<64>(), sizeof(TcmSmem<64>), s>>>(p, it);
    else if (p.m_tile == 256)
        wf_net_tcm_kernel<256, HH, false><<<n_sms * tcm_ctas_per_sm<256>(), tcm_threads<256>(), sizeof(TcmSmem<256>), s>>>(p, it);
    else wf_net_tc_kernel<0, HH, false><<<grid_tc, 128, tc_smem, s>>>(p, it);
}

template <bool CACHED, int HH>
static cudaError_t run_frame(const RenderParams &p, int n_sms, cudaStream_t s, int *h_pinned, int check_every, int *n_iter,
                             LaunchLog *log)
{
    {
        cudaError_t e = ensure_net_attrs<HH>();
        if (e != cudaSuccess) return e;
    }
    LaunchLog local;
    LaunchLog &L = log ? *log : local;
    auto timed_begin = [&]() {
        if (L.ev && L.n_timed < L.cap) cudaEventRecord(L.ev[2 * L.n_timed], s);
    };
    auto timed_end = [&]() {
        if (L.ev && L.n_timed < L.cap) cudaEventRecord(L.ev[2 * L.n_timed++ + 1], s);
        else if (L.ev) ++L.n_untimed;
    };
    const int W = p.cam.W, H = p.cam.H;
    const int n_threads = ((W + 7) / 8) * ((H + 3) / 4) * 32;
    if (p.pixel_list) wf_raygen_list_kernel<<<(p.n_list + 255) / 256, 256, 0, s>>>(p);
    else wf_raygen_kernel<<<(n_threads + 255) / 256, 256, 0, s>>>(p);
    ++L.launches;
    const int grid_ray = n_sms * FVC_RAY_BLOCKS_PER_SM;
    const int grid_net = n_sms * 2;
    const size_t net_smem = sizeof(NetSmem);
    const size_t tc_smem = tc_smem_bytes(p.freq);
    const int grid_tc = n_sms * FVC_TC_CTAS_PER_SM; /* <= 8 CTAs x 64 TMEM columns per SM */
    const bool fused = CACHED && fused_cached_path(p);
    int it = 0;
    const int max_it = 1 << 20;
    for (; it < max_it; ++it) {
        if (fused) {
            wf_march_kernel<true, true><<<grid_ray, 128, 0, s>>>(p, it);
            wf_cache_lookup_kernel<<<n_sms * 8, 256, 0, s>>>(p, it);
            timed_begin();
            wf_net_tc_kernel<2, HH, false><<<grid_tc, 128, tc_smem, s>>>(p, it);
            timed_end();
            L.launches += 3;
        } else {
            wf_march_kernel<CACHED><<<grid_ray, 128, 0, s>>>(p, it);
            ++L.launches;
        }
        if (CACHED && !fused) {
            launch_classify(p, it, n_sms, s);
            timed_begin();
            if (p.view_dependent) wf_net_vd_kernel<0, HH, true><<<n_sms * 4, 128, sizeof(VdSmem), s>>>(p, it);
            else if (p.use_tc) wf_net_tc_kernel<0, HH, true><<<grid_tc, 128, tc_smem, s>>>(p, it);
            else wf_net_resample_kernel<HH, true><<<grid_net, NET_WARPS * 32, net_smem, s>>>(p, it);
            timed_end();
            if (p.view_dependent) wf_net_vd_kernel<1, HH, true><<<n_sms * 4, 128, sizeof(VdSmem), s>>>(p, it);
            else if (p.use_tc) wf_net_tc_kernel<1, HH, true><<<grid_tc, 128, tc_smem, s>>>(p, it);
            else wf_net_cache_kernel<HH><<<grid_net, NET_WARPS * 32, net_smem, s>>>(p, it);
            L.launches += 3;
        } else if (!CACHED) {
            timed_begin();
            launch_plain_net<HH>(p, it, n_sms, s);
            timed_end();
            L.launches += 1;
        }
        wf_composite_kernel<CACHED><<<grid_ray, 128, 0, s>>>(p, it);
        wf_reset_rows_kernel<<<1, 32, 0, s>>>(p, CACHED ? 1 : 0);
        L.launches += 2;
        if ((it + 1) % check_every == 0) {
            cudaError_t e = cudaMemcpyAsync(h_pinned, p.counters + ((it + 1) & 1), sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) return e;
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return e;
            if (*h_pinned == 0) { ++it; break; }
        }
    }
    if (n_iter) *n_iter = it;
    return cudaGetLastError();
}

/* Self-test of the exact division (div_rn_by with the correctly rounded
 * reciprocal) against the hardware IEEE division, element by element. */
__global__ void div_selftest_kernel(const float *x, const float *d, int n, float *q, float *ieee)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i] = div_rn_by(x[i], d[i], __frcp_rn(d[i]));
    ieee[i] = __fdiv_rn(x[i], d[i]);
}

cudaError_t launch_div_selftest(const float *x, const float *d, int n, float *q, float *ieee)
{
    div_selftest_kernel<<<(n + 255) / 256, 256>>>(x, d, n, q, ieee);
    return cudaDeviceSynchronize();
}

/* Self-test of the bounded device wait: one warp waits on an mbarrier that
 * nothing arrives at; mbar_wait gives up after limit_cycles SM clocks and the
 * kernel reports it (out[0] = 1 when the wait ran out, out[1] = the cycles
 * waited) instead of hanging. */
__global__ void __launch_bounds__(32) wait_selftest_kernel(long long limit_cycles, long long *out)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const long long t0 = clock64();
    const bool ok = mbar_wait(&bar, 0, limit_cycles);
    const long long t1 = clock64();
    if (threadIdx.x == 0) {
        out[0] = ok ? 0 : 1;
        out[1] = t1 - t0;
    }
}

cudaError_t launch_wait_selftest(long long limit_cycles, long long *d_out, cudaStream_t s)
{
    wait_selftest_kernel<<<1, 32, 0, s>>>(limit_cycles, d_out);
    return cudaGetLastError();
}

/* the plain renderer's raygen and march, for the per-ray cache fill */
cudaError_t launch_fill_raygen(const RenderParams &p, cudaStream_t s)
{
    const int n_threads = ((p.cam.W + 7) / 8) * ((p.cam.H + 3) / 4) * 32;
    wf_raygen_kernel<<<(n_threads + 255) / 256, 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_fill_march(const RenderParams &p, int it, int n_sms, cudaStream_t s)
{
    wf_march_kernel<false><<<n_sms * FVC_RAY_BLOCKS_PER_SM, 128, 0, s>>>(p, it);
    return cudaGetLastError();
}

/* Pass 2 of the differentiable render (pass 1 is run_frame over the pixel
 * list, then the loss kernel): the same march and network forward per
 * sub-iteration, then the compositing adjoint and the network adjoint. */
template <bool CACHED, int HH>
static cudaError_t run_backward(const RenderParams &p, const BwdParams &b, int n_sms, cudaStream_t s, int *h_pinned,
                                int check_every, LaunchLog *log)
{
    {
        cudaError_t e = ensure_net_attrs<HH>();
        if (e != cudaSuccess) return e;
    }
    LaunchLog local;
    LaunchLog &L = log ? *log : local;
    wf_raygen_list_kernel<<<(p.n_list + 255) / 256, 256, 0, s>>>(p);
    ++L.launches;
    /* the network adjoint's launches are timed (when the renderer's kernel timing is on) */
    auto timed_begin = [&]() {
        if (L.ev && L.n_timed < L.cap) cudaEventRecord(L.ev[2 * L.n_timed], s);
    };
    auto timed_end = [&]() {
        if (L.ev && L.n_timed < L.cap) cudaEventRecord(L.ev[2 * L.n_timed++ + 1], s);
        else if (L.ev) ++L.n_untimed;
    };
    const int grid_ray = n_sms * FVC_RAY_BLOCKS_PER_SM;
    for (int it = 0; it < (1 << 20); ++it) {
        wf_march_kernel<CACHED><<<grid_ray, 128, 0, s>>>(p, it);
        /* the forward kernels of pass 1, so both passes composite the same values */
        if (CACHED) {
            const size_t tc_smem = tc_smem_bytes(p.freq);
            const int grid_tc = n_sms * FVC_TC_CTAS_PER_SM;
            launch_classify(p, it, n_sms, s);
            if (p.use_tc) {
                wf_net_tc_kernel<0, HH, true><<<grid_tc, 128, tc_smem, s>>>(p, it);
                wf_net_tc_kernel<1, HH, true><<<grid_tc, 128, tc_smem, s>>>(p, it);
            } else {
                wf_net_resample_kernel<HH, true><<<n_sms * 2, NET_WARPS * 32, sizeof(NetSmem), s>>>(p, it);
                wf_net_cache_kernel<HH><<<n_sms * 2, NET_WARPS * 32, sizeof(NetSmem), s>>>(p, it);
            }
            L.launches += 3;
        } else {
            launch_plain_net<HH>(p, it, n_sms, s);
            L.launches += 1;
        }
        wf_composite_bwd_kernel<CACHED><<<grid_ray, 128, 0, s>>>(p, it);
        timed_begin();
        cudaError_t e = launch_net_backward(p, b, HH, it, n_sms, s);
        timed_end();
        if (e == cudaSuccess && CACHED) e = launch_cache_backward(p, b, HH, it, n_sms, s);
        if (e != cudaSuccess) return e;
        wf_reset_rows_kernel<<<1, 32, 0, s>>>(p, CACHED ? 1 : 0);
        L.launches += CACHED ? 5 : 4;
        if ((it + 1) % check_every == 0) {
            e = cudaMemcpyAsync(h_pinned, p.counters + ((it + 1) & 1), sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e != cudaSuccess) return e;
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return e;
            if (*h_pinned == 0) break;
        }
    }
    return cudaGetLastError();
}

cudaError_t backward_frame(const RenderParams &p, const BwdParams &b, bool cached, int head_hidden, int n_sms, cudaStream_t s,
                           int *h_pinned, int check_every, LaunchLog *log)
{
    if (cached)
        return head_hidden == 2 ? run_backward<true, 2>(p, b, n_sms, s, h_pinned, check_every, log)
                                : run_backward<true, 1>(p, b, n_sms, s, h_pinned, check_every, log);
    return head_hidden == 2 ? run_backward<false, 2>(p, b, n_sms, s, h_pinned, check_every, log)
                            : run_backward<false, 1>(p, b, n_sms, s, h_pinned, check_every, log);
}

template <bool CACHED, int HH>
static cudaError_t build_batch_graph_t(const RenderParams &p, int n_sms, cudaStream_t s, int n_rays, cudaGraphExec_t *exec,
                                       int *n_kernels)
{
    {
        cudaError_t e = ensure_net_attrs<HH>();
        if (e != cudaSuccess) return e;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaGraphCreate(&graph, 0);
    if (e != cudaSuccess) return e;
    cudaGraphConditionalHandle handle;
    e = cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault);
    /* prologue: counters, statistics, raygen */
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaMemsetAsync(p.ray_counter, 0, 4 * sizeof(int), s);
        cudaMemsetAsync(p.stats, 0, sizeof(RenderStatsDev), s);
        cudaMemsetAsync(p.counters, 0, 8 * sizeof(int), s);
        wf_raygen_views_kernel<<<(n_rays + 255) / 256, 256, 0, s>>>(p);
        cudaGraph_t g2 = nullptr;
        e = cudaStreamEndCapture(s, &g2);
    }
    /* the loop: a WHILE node after the prologue's last node */
    cudaGraphNode_t prologue_tail = nullptr;
    if (e == cudaSuccess) {
        size_t n = 0;
        e = cudaGraphGetNodes(graph, nullptr, &n);
        std::vector<cudaGraphNode_t> nodes(n);
        if (e == cudaSuccess) e = cudaGraphGetNodes(graph, nodes.data(), &n);
        for (cudaGraphNode_t nd : nodes) { /* the node nothing depends on */
            size_t nout = 0;
            if (cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nout) == cudaSuccess && nout == 0) prologue_tail = nd;
        }
    }
    cudaGraphNode_t loop = nullptr;
    cudaGraph_t body = nullptr;
    if (e == cudaSuccess) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        e = cudaGraphAddNode(&loop, graph, &prologue_tail, nullptr, prologue_tail ? 1 : 0, &cp);
        if (e == cudaSuccess) body = cp.conditional.phGraph_out[0];
    }
    int kernels = 1;
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const int grid_ray = n_sms * FVC_RAY_BLOCKS_PER_SM;
        const bool fused = CACHED && fused_cached_path(p);
        for (int it = 0; it < 2; ++it) {
            if (fused) {
                wf_march_kernel<true, true><<<grid_ray, 128, 0, s>>>(p, it);
                wf_cache_lookup_kernel<<<n_sms * 8, 256, 0, s>>>(p, it);
                wf_net_tc_kernel<2, HH, false><<<n_sms * FVC_TC_CTAS_PER_SM, 128, tc_smem_bytes(p.freq), s>>>(p, it);
                kernels += 2;
            } else {
                wf_march_kernel<CACHED><<<grid_ray, 128, 0, s>>>(p, it);
            }
            if (CACHED && !fused) {
                const size_t tc_smem = tc_smem_bytes(p.freq);
                const int grid_tc = n_sms * FVC_TC_CTAS_PER_SM;
                launch_classify(p, it, n_sms, s);
                if (p.view_dependent) {
                    wf_net_vd_kernel<0, HH, true><<<n_sms * 4, 128, sizeof(VdSmem), s>>>(p, it);
                    wf_net_vd_kernel<1, HH, true><<<n_sms * 4, 128, sizeof(VdSmem), s>>>(p, it);
                } else if (p.use_tc) {
                    wf_net_tc_kernel<0, HH, true><<<grid_tc, 128, tc_smem, s>>>(p, it);
                    wf_net_tc_kernel<1, HH, true><<<grid_tc, 128, tc_smem, s>>>(p, it);
                } else {
                    wf_net_resample_kernel<HH, true><<<n_sms * 2, NET_WARPS * 32, sizeof(NetSmem), s>>>(p, it);
                    wf_net_cache_kernel<HH><<<n_sms * 2, NET_WARPS * 32, sizeof(NetSmem), s>>>(p, it);
                }
                kernels += 3;
            } else if (!CACHED) {
                launch_plain_net<HH>(p, it, n_sms, s);
                kernels += 1;
            }
            wf_composite_kernel<CACHED><<<grid_ray, 128, 0, s>>>(p, it);
            wf_reset_rows_kernel<<<1, 32, 0, s>>>(p, CACHED ? 1 : 0);
            kernels += 3;
        }
        wf_loop_cond_kernel<<<1, 1, 0, s>>>(p, handle);
        kernels += 1;
        cudaGraph_t g3 = nullptr;
        e = cudaStreamEndCapture(s, &g3);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (n_kernels) *n_kernels = kernels;
    return e;
}

cudaError_t build_batch_graph(const RenderParams &p, bool cached, int head_hidden, int n_sms, cudaStream_t s, int n_rays,
                              cudaGraphExec_t *exec, int *n_kernels)
{
    if (cached)
        return head_hidden == 2 ? build_batch_graph_t<true, 2>(p, n_sms, s, n_rays, exec, n_kernels)
                                : build_batch_graph_t<true, 1>(p, n_sms, s, n_rays, exec, n_kernels);
    return head_hidden == 2 ? build_batch_graph_t<false, 2>(p, n_sms, s, n_rays, exec, n_kernels)
                            : build_batch_graph_t<false, 1>(p, n_sms, s, n_rays, exec, n_kernels);
}

cudaError_t render_frame(const RenderParams &p, bool cached, int head_hidden, int n_sms, cudaStream_t s, int *h_pinned,
                         int check_every, int *n_iterations, LaunchLog *log)
{
    if (cached)
        return head_hidden == 2 ? run_frame<true, 2>(p, n_sms, s, h_pinned, check_every, n_iterations, log)
                                : run_frame<true, 1>(p, n_sms, s, h_pinned, check_every, n_iterations, log);
    return head_hidden == 2 ? run_frame<false, 2>(p, n_sms, s, h_pinned, check_every, n_iterations, log)
                            : run_frame<false, 1>(p, n_sms, s, h_pinned, check_every, n_iterations, log);
}

}  // namespace fvc
