/*
 * fvc_kernels.cu - the renderer's CUDA kernels for sm_103a.
 *
 *  render_kernel<CACHED>   persistent, warp-synchronous renderer.  Each warp
 *                          owns 32 rays (one per lane) and runs rounds of
 *                          (refill rays from a global queue, lockstep march
 *                          into an on-chip sample list, network on 32-row
 *                          batches on the tensor cores, in-order compositing).
 *                          Plain: PerformanceRenderer::render,
 *                          src/performance_renderer.cu:15-149,214-286.
 *                          Cached: CachePerformanceRenderer::render,
 *                          src/cache_performance_renderer.cu:22-313,678-908.
 *  cache_*_kernel          frustum cache build, one depth brick of every alive
 *                          8x8 tile per iteration with deterministic slots:
 *                          CacheRenderer::initCacheBlockwise,
 *                          src/cache_renderer.cu:18-569,931-1051.
 *  inference_kernel        network at given inputs (NerfNetwork::inference).
 *
 * Every loop is bounded; guards set bits in a device word instead of
 * trapping.
 */
#include "fvc_kernels.h"

#include <cuda_fp16.h>

namespace fvc {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() { unsigned m; asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m)); return m; }

/* voxel of the cache data array: density, isset, 2 pad words, 8 fp16 latents */
struct __align__(16) Voxel {
    float density, isset, pad0, pad1;
    uint4 lat;
};

/* ------------------------------------------------------------------------- */
/* render kernel                                                             */
/* ------------------------------------------------------------------------- */
constexpr int RK_WARPS = 8;       /* warps per CTA */
constexpr int KMAX = 4;           /* samples per lane per round */
constexpr int ROWS = 32 * KMAX;   /* resample rows from the front, cache rows from the back */
constexpr int ROUND_STEP_CAP = 256;
constexpr int ROW_TARGET = 96;

struct WarpSmem {
    float4 rows[ROWS];                 /* pos or froxel point, .w = lane | seq<<8 */
    __half tile[32 * TILE_STRIDE];
    float comp_t0[KMAX][32];
    uint2 comp_out[KMAX][32];          /* half logits r,g,b, half log-density */
    uint8_t comp_kind[KMAX][32];       /* 0 resample, 1 cache */
    float3 dir01[32];
};

struct RenderSmem {
    uint2 W[W_TOTAL];
    float bias3[64];
    WarpSmem warp[RK_WARPS];
};

__device__ __forceinline__ void write_pixel(const RenderParams &p, int ray, float r, float g, float b, float T, int4 counts)
{
    if (p.results) p.results[ray] = make_float4(r, g, b, T);
    if (p.ray_counts) p.ray_counts[ray] = counts;
    if (p.image) {
        /* writeImageBuffer_performance_kernel, src/performance_renderer.cu:127-149 */
        float cr = r + T, cg = g + T, cb = b + T;
        if (p.sample_index > 0) {
            const uchar4 prev = p.image[ray];
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
        p.image[ray] = o;
    }
}

/* cache texel (X,Y,Z) of the data array -> voxel pointer (or null outside:
 * border addressing returns zeros) */
__device__ __forceinline__ const Voxel *texel(const CacheView &c, int X, int Y, int Z)
{
    if (X < 0 || Y < 0 || Z < 0 || X >= c.dX * 8 || Y >= c.dY * 8 || Z >= c.dZ * 8) return nullptr;
    const int slot = (X >> 3) * (c.dY * c.dZ) + (Y >> 3) * c.dZ + (Z >> 3);
    if (slot >= c.n_valid_slots) return nullptr; /* the reference clears the data arrays per build */
    return reinterpret_cast<const Voxel *>(c.voxels) + (size_t)slot * 512 + ((Z & 7) * 64 + (Y & 7) * 8 + (X & 7));
}

template <bool CACHED, int HEAD_HIDDEN>
__global__ void __launch_bounds__(RK_WARPS * 32, 2) render_kernel(RenderParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RenderSmem &S = *reinterpret_cast<RenderSmem *>(smem_raw);
    for (int i = threadIdx.x; i < W_TOTAL; i += blockDim.x) S.W[i] = p.weights[i];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) S.bias3[i] = p.bias3[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    WarpSmem &ws = S.warp[threadIdx.x >> 5];
    const int n_rays = p.cam.W * p.cam.H;

    int ray = -1;
    float3 o = make_float3(0, 0, 0), d = make_float3(0, 0, 0), oc = o, dc = o;
    float far_ = 0.f, t1 = 0.f, cr = 0.f, cg = 0.f, cb = 0.f, T = 1.f;
    bool done = false, term = false;
    int nsamp = 0, c_res = 0, c_cache = 0, c_drop = 0, c_steps = 0;
    bool exhausted = false;
    long long st_samples = 0, st_res = 0, st_cache = 0, st_drop = 0, st_steps = 0;
    int rounds = 0;

    for (int round = 0; round < p.max_rounds; ++round) {
        /* ---- refill lanes from the ray queue ---- */
        for (int it = 0; it < 64 && !exhausted; ++it) {
            const unsigned need = __ballot_sync(FULL, ray < 0);
            if (need == 0) break;
            int base = 0;
            if (lane == 0) base = atomicAdd(p.ray_counter, __popc(need));
            base = __shfl_sync(FULL, base, 0);
            if (base + __popc(need) >= n_rays) exhausted = true;
            if (ray < 0) {
                const int id = base + __popc(need & lanemask_lt());
                if (id < n_rays) {
                    const int x = id % p.cam.W, y = id / p.cam.W;
                    generate_ray(p.cam, x, y, o, d);
                    float tn, tf;
                    const bool hits = ray_aabb(o, d, p.scene.aabb_from, p.scene.aabb_to, tn, tf);
                    if (!hits) {
                        write_pixel(p, id, 0.f, 0.f, 0.f, 1.f, make_int4(0, 0, 0, 0));
                    } else {
                        ray = id;
                        far_ = fminf(tf, p.steps.far_);
                        t1 = F_ADD(valid_t_from_t(p.steps, tn), 0.0f);
                        cr = cg = cb = 0.f; T = 1.f; done = false; term = false;
                        nsamp = c_res = c_cache = c_drop = c_steps = 0;
                        if (CACHED) transform_ray(p.ccam.w2c, o, d, oc, dc);
                        ws.dir01[lane] = make_float3(F_DIV(F_ADD(d.x, 1.0f), 2.0f), F_DIV(F_ADD(d.y, 1.0f), 2.0f),
                                                     F_DIV(F_ADD(d.z, 1.0f), 2.0f));
                    }
                }
            }
        }
        if (__ballot_sync(FULL, ray >= 0) == 0) break;
        ++rounds;

        /* ---- lockstep march into the sample list ---- */
        int n_res = 0, n_cache = 0, k = 0;
        for (int it = 0; it < ROUND_STEP_CAP; ++it) {
            const bool act = ray >= 0 && !done && k < KMAX;
            if (!__any_sync(FULL, act) || n_res + n_cache >= ROW_TARGET) break;
            int kind = -1;
            float3 rv = make_float3(0.f, 0.f, 0.f);
            float t0 = 0.f;
            if (act) {
                t0 = t1;
                const float dt = calc_step(p.steps, t0);
                t1 = F_ADD(t0, dt);
                const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
                ++st_steps;
                ++c_steps;
                if (tm > far_) {
                    done = true;
                } else {
                    const float3 wp = at(o, d, tm);
                    if (occupied(p.scene, p.bits, wp)) {
                        if (!CACHED) {
                            kind = 0;
                            rv = contract(p.scene, wp);
                        } else {
                            /* classification, sample_cache_performance_kernel :91-163 */
                            float tfr;
                            const float3 fr = cam2froxel(at(oc, dc, tm), p.ccam, p.csteps, tfr);
                            const CacheView &C = p.cache;
                            const bool in_fov = fr.x >= 0.f && fr.x < (float)C.fW && fr.y >= 0.f && fr.y < (float)C.fH;
                            const bool inside = in_fov && fr.z >= 0.f && fr.z < (float)C.fD;
                            bool unsampled = true;
                            if (in_fov) {
                                const float kr = __ldg(C.known_ranges + (size_t)(int)floorf(fr.y) * C.fW + (int)floorf(fr.x));
                                unsampled = tfr < p.csteps.near_ || tfr > kr;
                            }
                            const float tmh = F_ADD(t0, F_MUL(dt, 0.5f));  /* generateNetworkInput_*: t0 + dt/2 */
                            if (!inside || unsampled) {
                                if (p.render_mode != 1) { kind = 0; rv = contract(p.scene, at(o, d, tmh)); }
                            } else if (p.render_mode != 2) {
                                const int bx = (int)F_DIV(fr.x, 8.0f), by = (int)F_DIV(fr.y, 8.0f), bz = (int)F_DIV(fr.z, 8.0f);
                                const int packed = __ldg(C.packed_index + ((size_t)bz * C.bY + by) * C.bX + bx);
                                kind = 2;
                                if (packed >= 0) {
                                    const float ax = F_ADD((float)(((packed >> 20) & 1023) * 8), F_SUB(fr.x, (float)(bx * 8)));
                                    const float ay = F_ADD((float)(((packed >> 10) & 1023) * 8), F_SUB(fr.y, (float)(by * 8)));
                                    const float az = F_ADD((float)((packed & 1023) * 8), F_SUB(fr.z, (float)(bz * 8)));
                                    const Voxel *v = texel(C, (int)floorf(ax), (int)floorf(ay), (int)floorf(az));
                                    if (v && __ldg(&v->density) > 0.0f) {
                                        kind = 1;
                                        float tf2;
                                        rv = cam2froxel(at(oc, dc, tmh), p.ccam, p.csteps, tf2);
                                    }
                                }
                                if (kind == 2) { ++st_drop; ++c_drop; }
                            }
                        }
                    }
                }
            }
            const unsigned m0 = __ballot_sync(FULL, kind == 0), m1 = __ballot_sync(FULL, kind == 1);
            if (kind == 0 || kind == 1) {
                const int idx = kind == 0 ? n_res + __popc(m0 & lanemask_lt()) : ROWS - 1 - (n_cache + __popc(m1 & lanemask_lt()));
                ws.rows[idx] = make_float4(rv.x, rv.y, rv.z, __int_as_float(lane | (k << 8)));
                ws.comp_t0[k][lane] = t0;
                ws.comp_kind[k][lane] = (uint8_t)kind;
                ++k;
                if (++nsamp > p.max_samples_per_ray && p.max_samples_per_ray > 0) atomicOr(p.guard, 1);
            }
            n_res += __popc(m0);
            n_cache += __popc(m1);
        }
        __syncwarp();
        st_res += n_res;
        st_cache += n_cache;

        /* ---- resample rows: hash grid + density net + color head ---- */
        for (int b = 0; b < n_res; b += 32) {
            const int r = b + lane;
            __half *trow = ws.tile + lane * TILE_STRIDE;
            if (r < n_res) {
                const float4 rw = ws.rows[r];
                hash_encode(p.grid, p.table, make_float3(rw.x, rw.y, rw.z), reinterpret_cast<__half2 *>(trow));
                sh16(ws.dir01[__float_as_int(rw.w) & 31], reinterpret_cast<__half2 *>(trow + 32));
            } else {
                for (int c = 0; c < 24; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
            }
            __syncwarp();
            density_mlp(ws.tile, S.W, lane);
            float lo[2][4];
            color_mlp<HEAD_HIDDEN>(ws.tile, S.W, S.bias3, lane, lo);
            {
                const int g = lane >> 2, t = lane & 3;
                if (t < 2) {
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) {
                        __half *r0 = ws.tile + (16 * mt + g) * TILE_STRIDE + 48 + 2 * t;
                        *reinterpret_cast<uint32_t *>(r0) = pack_h2(lo[mt][0], lo[mt][1]);
                        *reinterpret_cast<uint32_t *>(r0 + 8 * TILE_STRIDE) = pack_h2(lo[mt][2], lo[mt][3]);
                    }
                }
            }
            __syncwarp();
            if (r < n_res) {
                const int tag = __float_as_int(ws.rows[r].w);
                const uint32_t rg = *reinterpret_cast<const uint32_t *>(trow + 48);
                const uint32_t bs = (uint32_t)__half_as_ushort(trow[50]) | ((uint32_t)__half_as_ushort(trow[16]) << 16);
                ws.comp_out[tag >> 8][tag & 31] = make_uint2(rg, bs);
            }
            __syncwarp();
        }

        /* ---- cache rows: trilinear lookup + color head ---- */
        if (CACHED) {
            for (int b = 0; b < n_cache; b += 32) {
                const int r = b + lane;
                __half *trow = ws.tile + lane * TILE_STRIDE;
                if (r < n_cache) {
                    const float4 rw = ws.rows[ROWS - 1 - r];
                    const CacheView &C = p.cache;
                    /* generateNetworkInput_cache_shfl_perf_kernel_cg :678-787 */
                    const float fx = F_SUB(rw.x, 0.5f), fy = F_SUB(rw.y, 0.5f), fz = F_SUB(rw.z, 0.5f);
                    const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
                    const float lx = F_SUB(fx, x0), ly = F_SUB(fy, y0), lz = F_SUB(fz, z0);
                    float wsum = 0.f, dsum = 0.f, ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
                        const float cx = x0 + (float)ox, cy = y0 + (float)oy, cz = z0 + (float)oz;
                        const bool inside = cx >= 0.f && cx < (float)C.fW && cy >= 0.f && cy < (float)C.fH && cz >= 0.f && cz < (float)C.fD;
                        if (!inside) continue;
                        const int bx = (int)F_DIV(cx, 8.0f), by = (int)F_DIV(cy, 8.0f), bz = (int)F_DIV(cz, 8.0f);
                        const int packed = __ldg(C.packed_index + ((size_t)bz * C.bY + by) * C.bX + bx);
                        if (packed < 0) continue;
                        const Voxel *v = texel(C, ((packed >> 20) & 1023) * 8 + ((int)cx - bx * 8),
                                               ((packed >> 10) & 1023) * 8 + ((int)cy - by * 8), (packed & 1023) * 8 + ((int)cz - bz * 8));
                        if (!v) continue;
                        const float w = (ox ? lx : 1.0f - lx) * (oy ? ly : 1.0f - ly) * (oz ? lz : 1.0f - lz);
                        const float2 di = __ldg(reinterpret_cast<const float2 *>(v));
                        const uint4 lt = __ldg(&v->lat);
                        wsum = fmaf(w, di.y, wsum);
                        dsum = fmaf(w, di.x, dsum);
                        const uint32_t lw[4] = {lt.x, lt.y, lt.z, lt.w};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&lw[q]));
                            ls[2 * q] = fmaf(w, f.x, ls[2 * q]);
                            ls[2 * q + 1] = fmaf(w, f.y, ls[2 * q + 1]);
                        }
                    }
                    uint32_t *hin = reinterpret_cast<uint32_t *>(trow + 16);
                    for (int c = 0; c < 8; ++c) hin[c] = 0u;
                    trow[16] = __float2half_rn(logf(fmaxf(dsum, 1e-6f)));
                    const float inv = 1.0f / wsum;
#pragma unroll
                    for (int j = 0; j < 8; ++j) trow[16 + p.latent_offset + j] = __float2half_rn(ls[j] * inv);
                    sh16(ws.dir01[__float_as_int(rw.w) & 31], reinterpret_cast<__half2 *>(trow + 32));
                } else {
                    for (int c = 8; c < 24; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
                }
                __syncwarp();
                float lo[2][4];
                color_mlp<HEAD_HIDDEN>(ws.tile, S.W, S.bias3, lane, lo);
                {
                    const int g = lane >> 2, t = lane & 3;
                    if (t < 2) {
#pragma unroll
                        for (int mt = 0; mt < 2; ++mt) {
                            __half *r0 = ws.tile + (16 * mt + g) * TILE_STRIDE + 48 + 2 * t;
                            *reinterpret_cast<uint32_t *>(r0) = pack_h2(lo[mt][0], lo[mt][1]);
                            *reinterpret_cast<uint32_t *>(r0 + 8 * TILE_STRIDE) = pack_h2(lo[mt][2], lo[mt][3]);
                        }
                    }
                }
                __syncwarp();
                if (r < n_cache) {
                    const int tag = __float_as_int(ws.rows[ROWS - 1 - r].w);
                    const uint32_t rg = *reinterpret_cast<const uint32_t *>(trow + 48);
                    const uint32_t bs = (uint32_t)__half_as_ushort(trow[50]) | ((uint32_t)__half_as_ushort(trow[16]) << 16);
                    ws.comp_out[tag >> 8][tag & 31] = make_uint2(rg, bs);
                }
                __syncwarp();
            }
        }

        /* ---- in-order compositing, accumulate_performance_kernel
         *      (src/performance_renderer.cu:93-121) ---- */
        for (int s = 0; s < k && !term; ++s) {
            const float t0 = ws.comp_t0[s][lane];
            const uint2 ov = ws.comp_out[s][lane];
            const float2 rg = __half22float2(*reinterpret_cast<const __half2 *>(&ov.x));
            const float lb = __half2float(__ushort_as_half((unsigned short)(ov.y & 0xffffu)));
            const float ld = __half2float(__ushort_as_half((unsigned short)(ov.y >> 16)));
            const float dt = calc_step(p.steps, t0);
            if (ws.comp_kind[s][lane]) ++c_cache; else ++c_res;
            const float sigma = expf(ld);
            const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-sigma * dt)));
            if (alpha > p.scene.alpha_thre) {
                const float w = alpha * T;
                cr += w / (1.0f + expf(-rg.x));
                cg += w / (1.0f + expf(-rg.y));
                cb += w / (1.0f + expf(-lb));
                T *= 1.0f - alpha;
            }
            if (T < 1e-4f) term = true;
        }
        st_samples += k;
        __syncwarp();

        /* ---- finish rays ---- */
        if (ray >= 0 && (done || term)) {
            write_pixel(p, ray, cr, cg, cb, T, make_int4(c_res, c_cache, c_drop, c_steps));
            ray = -1;
        }
    }
    if (ray >= 0) atomicOr(p.guard, 2); /* round limit reached with a ray in flight */

    /* statistics: one atomic per warp */
    const long long wsamp = __reduce_add_sync(FULL, (unsigned)st_samples);
    const long long wres = __reduce_add_sync(FULL, (unsigned)st_res);
    const long long wcache = __reduce_add_sync(FULL, (unsigned)st_cache);
    const long long wdrop = __reduce_add_sync(FULL, (unsigned)st_drop);
    const long long wsteps = __reduce_add_sync(FULL, (unsigned)st_steps);
    if (lane == 0) {
        atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->n_samples), (unsigned long long)wsamp);
        atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->n_resamples), (unsigned long long)(CACHED ? wres : wsamp));
        atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->n_cache_hits), (unsigned long long)wcache);
        atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->n_dropped), (unsigned long long)wdrop);
        atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->n_steps), (unsigned long long)wsteps);
        atomicMax(&p.stats->n_rounds, rounds);
    }
}

size_t render_smem_bytes() { return sizeof(RenderSmem); }

template <bool CACHED, int HH>
static cudaError_t launch_render_t(const RenderParams &p, int n_sms, cudaStream_t s)
{
    auto kern = render_kernel<CACHED, HH>;
    const size_t smem = sizeof(RenderSmem);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RK_WARPS * 32, smem);
    if (e != cudaSuccess) return e;
    const int grid = max(1, per_sm) * n_sms;
    kern<<<grid, RK_WARPS * 32, smem, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_render(const RenderParams &p, bool cached, int head_hidden, int n_sms, cudaStream_t s)
{
    if (cached) return head_hidden == 2 ? launch_render_t<true, 2>(p, n_sms, s) : launch_render_t<true, 1>(p, n_sms, s);
    return head_hidden == 2 ? launch_render_t<false, 2>(p, n_sms, s) : launch_render_t<false, 1>(p, n_sms, s);
}

/* ------------------------------------------------------------------------- */
/* network at given inputs (testing / occupancy generation)                   */
/* ------------------------------------------------------------------------- */
template <int HEAD_HIDDEN>
__global__ void __launch_bounds__(128) inference_kernel(InferenceParams p)
{
    __shared__ uint2 Wsm[W_TOTAL];
    __shared__ float bsm[64];
    __shared__ __align__(16) __half tiles[4][32 * TILE_STRIDE];
    for (int i = threadIdx.x; i < W_TOTAL; i += blockDim.x) Wsm[i] = p.weights[i];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) bsm[i] = p.bias3[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __half *tile = tiles[w];
    const int n_batches = (p.n + 31) / 32;
    for (int b = blockIdx.x * 4 + w; b < n_batches; b += gridDim.x * 4) {
        const int r = b * 32 + lane;
        __half *trow = tile + lane * TILE_STRIDE;
        if (r < p.n) {
            const float3 pos = make_float3(p.pos[3 * r], p.pos[3 * r + 1], p.pos[3 * r + 2]);
            hash_encode(p.grid, p.table, pos, reinterpret_cast<__half2 *>(trow));
            if (p.features)
                for (int j = 0; j < 32; ++j) p.features[32 * r + j] = __half2float(trow[j]);
            if (p.dir) sh16(make_float3(p.dir[3 * r], p.dir[3 * r + 1], p.dir[3 * r + 2]), reinterpret_cast<__half2 *>(trow + 32));
        } else {
            for (int c = 0; c < 24; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
        }
        __syncwarp();
        density_mlp(tile, Wsm, lane);
        if (p.dir) {
            float lo[2][4];
            color_mlp<HEAD_HIDDEN>(tile, Wsm, bsm, lane, lo);
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
        __syncwarp();
        if (r < p.n) {
            if (p.out4) {
                p.out4[4 * r + 0] = p.dir ? __half2float(trow[48]) : 0.f;
                p.out4[4 * r + 1] = p.dir ? __half2float(trow[49]) : 0.f;
                p.out4[4 * r + 2] = p.dir ? __half2float(trow[50]) : 0.f;
                p.out4[4 * r + 3] = __half2float(trow[16]);
            }
            if (p.base_out)
                for (int j = 0; j < 16; ++j) p.base_out[16 * r + j] = __half2float(trow[16 + j]);
        }
        __syncwarp();
    }
}

cudaError_t launch_inference(const InferenceParams &p, int head_hidden, int n_sms, cudaStream_t s)
{
    const int n_batches = (p.n + 31) / 32;
    const int grid = max(1, min((n_batches + 3) / 4, n_sms * 8));
    if (head_hidden == 2) inference_kernel<2><<<grid, 128, 0, s>>>(p);
    else inference_kernel<1><<<grid, 128, 0, s>>>(p);
    return cudaGetLastError();
}

/* ------------------------------------------------------------------------- */
/* frustum cache build                                                       */
/* ------------------------------------------------------------------------- */

/* initPayloads_cache_init_kernel, src/cache_renderer.cu:18-81: one CTA of
 * 64 threads per 8x8 tile. */
__global__ void __launch_bounds__(64) cache_init_kernel(CacheBuildParams p)
{
    const int tile = blockIdx.x;
    const int k = threadIdx.x;
    const int tx = tile % p.bX, ty = tile / p.bX;
    const int px = tx * 8 + (k & 7), py = ty * 8 + (k >> 3);
    float3 o, d;
    generate_ray(p.cam, px, py, o, d);
    float tn, tf;
    const bool hits = ray_aabb(o, d, p.scene.aabb_from, p.scene.aabb_to, tn, tf);
    const int start_step = max(0, (int)F_SUB(step_from_t(p.steps, hits ? tn : p.steps.near_), p.steps.near_i));
    CacheRay cr;
    cr.o = o; cr.d = d;
    cr.far_ = hits ? fminf(tf, p.steps.far_) : p.steps.far_;
    cr.T = 1.0f;
    cr.alive = hits ? 1 : 0;
    p.rays[(size_t)tile * 64 + k] = cr;
    __shared__ int s_alive[2], s_min[2];
    const int wa = __reduce_add_sync(FULL, hits ? 1 : 0);
    const int wm = __reduce_min_sync(FULL, (unsigned)start_step);
    if ((k & 31) == 0) { s_alive[k >> 5] = wa; s_min[k >> 5] = wm; }
    __syncthreads();
    if (k == 0) {
        p.block_step[tile] = min(s_min[0], s_min[1]) / 8;
        p.tile_alive[tile] = (s_alive[0] + s_alive[1]) > 0;
    }
}

struct BuildSmem {
    uint2 W[W_L3];                /* density network weights only */
    float4 rows[512];             /* contracted position, .w = ray | step<<6 */
    __half tile[2][32 * TILE_STRIDE];
    __half out[512][9];           /* per row: log-density + 8 latents (fp16) */
    short row_of[64][8];          /* row index of (ray, step) or -1 */
    int red[4];
};

/* One depth brick per alive tile: sample_cache_init_first_kernel (search),
 * sample_cache_init_second_kernel (samples), inferenceLatents, and the
 * density-only compositing of accumulateNew_cache_init_second_kernel
 * (src/cache_renderer.cu:83-528).  The brick's voxels go to a staging area
 * indexed by the tile's position in the alive list; slots are assigned by
 * cache_assign_kernel afterwards. */
__global__ void __launch_bounds__(64) cache_tile_kernel(CacheBuildParams p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BuildSmem &S = *reinterpret_cast<BuildSmem *>(smem_raw);
    const int k = threadIdx.x, lane = k & 31, wid = k >> 5;
    for (int i = k; i < W_L3; i += 64) S.W[i] = p.weights[i];
    const int n_alive_tiles = *p.n_alive_tiles;
    for (int ai = blockIdx.x; ai < n_alive_tiles; ai += gridDim.x) {
        __syncthreads();
        const int tile = p.alive_list[ai];
        CacheRay cr = p.rays[(size_t)tile * 64 + k];
        int bstep = p.block_step[tile];
        auto block_sum = [&](int v) -> int {
            const int w = __reduce_add_sync(FULL, (unsigned)v);
            __syncthreads();
            if (lane == 0) S.red[wid] = w;
            __syncthreads();
            return S.red[0] + S.red[1];
        };
        /* ---- search for the next depth brick with an occupied sample ---- */
        int total = 0;
        uint32_t mask = 0;
        for (int guard = 0; guard < p.max_search; ++guard) {
            if (block_sum(cr.alive) <= 0) break;
            if (bstep >= p.bZ) { cr.alive = 0; total = 0; break; } /* beyond the frustum depth: stop the tile */
            const float t1s = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
            float t1 = t1s;
            mask = 0;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const float t0 = t1;
                const float dt = calc_step(p.steps, t0);
                t1 = F_ADD(t0, dt);
                const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
                if (tm > cr.far_) cr.alive = 0;
                else if (occupied(p.scene, p.bits, at(cr.o, cr.d, tm))) mask |= 1u << s;
            }
            total = block_sum(__popc(mask));
            if (total > 0) break;
            ++bstep;
            if (guard == p.max_search - 1) atomicOr(p.guard, 4);
        }
        const int n_alive = block_sum(cr.alive);
        const bool processed = total > 0 && n_alive > 0;
        if (k == 0) {
            p.tile_n_samples[ai] = total;
            p.tile_processed[ai] = processed;
            p.tile_alive[tile] = n_alive > 0;
            p.block_step[tile] = bstep;
        }
        if (!processed) {
            p.rays[(size_t)tile * 64 + k] = cr;
            continue;
        }
        /* ---- emit samples (compact over the tile) ---- */
        const int cnt = __popc(mask);
        int incl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, off);
            if (lane >= off) incl += v;
        }
        if (lane == 31) S.red[2 + wid] = incl;
        __syncthreads();
        int base = incl - cnt + (wid ? S.red[2] : 0);
        {
            float t1 = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const float t0 = t1;
                const float dt = calc_step(p.steps, t0);
                t1 = F_ADD(t0, dt);
                const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
                if ((mask >> s) & 1u) {
                    const float3 cp = contract(p.scene, at(cr.o, cr.d, tm));
                    S.rows[base] = make_float4(cp.x, cp.y, cp.z, __int_as_float(k | (s << 6)));
                    S.row_of[k][s] = (short)base;
                    ++base;
                } else {
                    S.row_of[k][s] = -1;
                }
            }
        }
        __syncthreads();
        /* ---- density network on 32-row batches (warp w: batches w, w+2, ...) ---- */
        __half *tile_w = S.tile[wid];
        for (int b = wid * 32; b < total; b += 64) {
            const int r = b + lane;
            __half *trow = tile_w + lane * TILE_STRIDE;
            if (r < total) {
                const float4 rw = S.rows[r];
                hash_encode(p.grid, p.table, make_float3(rw.x, rw.y, rw.z), reinterpret_cast<__half2 *>(trow));
            } else {
                for (int c = 0; c < 16; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
            }
            __syncwarp();
            density_mlp(tile_w, S.W, lane);
            if (r < total) {
                S.out[r][0] = trow[16];
#pragma unroll
                for (int j = 0; j < 8; ++j) S.out[r][1 + j] = trow[16 + p.latent_offset + j];
            }
            __syncwarp();
        }
        __syncthreads();
        /* ---- density-only compositing (accumulateNew_cache_init_second_kernel :349-393) ---- */
        int visible = 0;
        {
            float t1 = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
            float T = cr.T;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const float t0 = t1;
                const float dt = calc_step(p.steps, t0);
                t1 = F_ADD(t0, dt);
                const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
                if (tm > cr.far_) { cr.alive = 0; continue; }
                if (!((mask >> s) & 1u)) continue;
                const float sigma = expf(__half2float(S.out[S.row_of[k][s]][0]));
                const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-sigma * dt)));
                if (alpha > p.scene.alpha_thre) { T *= 1.0f - alpha; ++visible; }
                if (T < 1e-4f) cr.alive = 0;
            }
            cr.T = T;
        }
        const int n_visible = block_sum(visible);
        const int n_alive_post = block_sum(cr.alive);
        if (k == 0) {
            p.tile_need[ai] = n_visible > 0;
            p.tile_n_alive[ai] = n_alive_post;
        }
        p.rays[(size_t)tile * 64 + k] = cr;
        /* ---- staging: all 512 voxels of the brick (zeros where no sample) ---- */
        if (n_visible > 0) {
            Voxel *st = reinterpret_cast<Voxel *>(p.staging) + (size_t)ai * 512;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                Voxel v;
                const int r = S.row_of[k][s];
                if (r >= 0) {
                    v.density = expf(__half2float(S.out[r][0]));
                    v.isset = 1.0f;
                    uint32_t lw[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        lw[q] = (uint32_t)__half_as_ushort(S.out[r][1 + 2 * q]) | ((uint32_t)__half_as_ushort(S.out[r][2 + 2 * q]) << 16);
                    v.lat = make_uint4(lw[0], lw[1], lw[2], lw[3]);
                } else {
                    v.density = 0.f; v.isset = 0.f; v.lat = make_uint4(0, 0, 0, 0);
                }
                v.pad0 = v.pad1 = 0.f;
                st[s * 64 + k] = v;
            }
        }
    }
}

size_t build_smem_bytes() { return sizeof(BuildSmem); }

/* Exclusive scan over a 1024-thread block; *total receives the block sum.
 * s_w must hold 33 ints. */
__device__ __forceinline__ int block_exclusive_scan(int v, int &total, int *s_w)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int u = __shfl_up_sync(FULL, inc, off);
        if (lane >= off) inc += u;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int w = s_w[lane];
        int wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int u = __shfl_up_sync(FULL, wi, off);
            if (lane >= off) wi += u;
        }
        s_w[lane] = wi - w;
        if (lane == 31) s_w[32] = wi;
    }
    __syncthreads();
    const int excl = s_w[wid] + inc - v;
    total = s_w[32];
    __syncthreads();
    return excl;
}

/* Deterministic slot assignment for one iteration (replaces the atomicAdd of
 * accumulateNew_cache_init_second_kernel, src/cache_renderer.cu:419-426):
 * the tiles needing a brick get consecutive slots in alive-list (= tile
 * index) order.  Applies the per-tile updates of :518-527 (block step
 * advances unless the allocation overflowed; the tile stays alive while it
 * has alive rays and did not overflow), emits the staging->slot copy jobs and
 * the next alive list.  One CTA of 1024 threads. */
__global__ void __launch_bounds__(1024) cache_assign_kernel(CacheBuildParams p)
{
    __shared__ int s_w[33];
    __shared__ int s_slot, s_jobs, s_alive;
    const int tid = threadIdx.x;
    const int n = *p.n_alive_tiles;
    if (tid == 0) { s_slot = *p.slot_counter; s_jobs = 0; s_alive = 0; }
    __syncthreads();
    for (int c0 = 0; c0 < n; c0 += 1024) {
        const int ai = c0 + tid;
        const bool valid = ai < n;
        const int tile = valid ? p.alive_list[ai] : 0;
        const bool processed = valid && p.tile_processed[ai];
        const bool need = processed && p.tile_need[ai];
        int n_need;
        const int slot = s_slot + block_exclusive_scan(need ? 1 : 0, n_need, s_w);
        const bool overflow = need && slot >= p.capacity;
        bool alive_next = false;
        if (valid) {
            const int bstep = p.block_step[tile];
            if (processed) {
                if (need) {
                    const int tx = tile % p.bX, ty = tile / p.bX;
                    if (bstep < p.bZ) {
                        const size_t bidx = ((size_t)bstep * p.bY + ty) * p.bX + tx;
                        if (!overflow) {
                            const int sx = slot / (p.dY * p.dZ), sy = (slot - sx * p.dY * p.dZ) / p.dZ;
                            const int sz = slot - sx * p.dY * p.dZ - sy * p.dZ;
                            p.packed_index[bidx] = (sx << 20) | (sy << 10) | sz;  /* pack3D(to3D(slot)) */
                        } else {
                            p.packed_index[bidx] = -1;
                        }
                    } else {
                        atomicOr(p.guard, 8);  /* brick beyond the frustum depth */
                    }
                }
                p.block_step[tile] = bstep + (overflow ? 0 : 1);
                alive_next = !overflow && p.tile_n_alive[ai] > 0;
                p.tile_alive[tile] = alive_next;
            } else {
                alive_next = p.tile_alive[tile] != 0;
            }
        }
        const bool job = valid && need && !overflow;
        int n_job, n_al;
        const int jpos = s_jobs + block_exclusive_scan(job ? 1 : 0, n_job, s_w);
        const int apos = s_alive + block_exclusive_scan(alive_next ? 1 : 0, n_al, s_w);
        if (job) { p.jobs[2 * jpos] = ai; p.jobs[2 * jpos + 1] = slot; }
        if (alive_next) p.alive_list_next[apos] = tile;
        __syncthreads();
        if (tid == 0) { s_slot += n_need; s_jobs += n_job; s_alive += n_al; }
        __syncthreads();
    }
    if (tid == 0) {
        *p.slot_counter = s_slot;
        *p.n_jobs = s_jobs;
        *p.n_alive_next = s_alive;
    }
}

/* staging -> data array for the bricks that got a slot */
__global__ void __launch_bounds__(256) cache_copy_kernel(CacheBuildParams p)
{
    const int n_jobs = *p.n_jobs;
    for (int j = blockIdx.x; j < n_jobs; j += gridDim.x) {
        const int ai = p.jobs[2 * j], slot = p.jobs[2 * j + 1];
        const uint4 *src = reinterpret_cast<const uint4 *>(p.staging) + (size_t)ai * 1024;
        uint4 *dst = reinterpret_cast<uint4 *>(p.voxels) + (size_t)slot * 1024;
        for (int i = threadIdx.x; i < 1024; i += blockDim.x) dst[i] = __ldcs(src + i);
    }
}

/* writeImageBuffer_cache_init_kernel2, src/cache_renderer.cu:530-569:
 * known_ranges_to = t at the start of the tile's final depth brick. */
__global__ void __launch_bounds__(64) cache_known_ranges_kernel(CacheBuildParams p)
{
    const int tile = blockIdx.x, k = threadIdx.x;
    const int tx = tile % p.bX, ty = tile / p.bX;
    const int px = tx * 8 + (k & 7), py = ty * 8 + (k >> 3);
    if (px >= p.fW || py >= p.fH) return;
    p.known_ranges[(size_t)py * p.fW + px] = t_from_step(p.steps, F_ADD((float)(p.block_step[tile] * 8), p.steps.near_i));
}

/* compaction of the initially alive tiles (single CTA of 1024 threads) */
__global__ void __launch_bounds__(1024) cache_compact_kernel(CacheBuildParams p, int n_tiles)
{
    __shared__ int s_w[33];
    __shared__ int s_carry;
    const int tid = threadIdx.x;
    if (tid == 0) s_carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < n_tiles; c0 += 1024) {
        const int t = c0 + tid;
        const int a = (t < n_tiles && p.tile_alive[t]) ? 1 : 0;
        int total;
        const int pos = s_carry + block_exclusive_scan(a, total, s_w);
        if (a) p.alive_list[pos] = t;
        __syncthreads();
        if (tid == 0) s_carry += total;
        __syncthreads();
    }
    if (tid == 0) *p.n_alive_tiles = s_carry;
}

}  // namespace fvc
