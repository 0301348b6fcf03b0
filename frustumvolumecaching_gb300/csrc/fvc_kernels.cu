/*
 * fvc_kernels.cu - the renderer's CUDA kernels for sm_103a.
 *
 *  (the renderer's wavefront kernels live in fvc_render.cu)
 *  cache_*_kernel          frustum cache build, one depth brick of every alive
 *                          8x8 tile per iteration (search, density network,
 *                          compositing, then deterministic slots):
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

/* The blockwise cache build (CacheRenderer::initCacheBlockwise,
 * src/cache_renderer.cu:931-1051) as a wavefront per depth-brick iteration:
 *   cache_search_kernel    per alive tile: the next depth brick holding an
 *                          occupied sample, its samples appended to a row list
 *                          (sample_cache_init_first/second_kernel :83-287);
 *   cache_density_kernel   the density network on all rows of the iteration
 *                          (inferenceLatents), warp-level tensor-core MLP;
 *   cache_composite_kernel per processed tile: density-only compositing and
 *                          the brick's need of a slot
 *                          (accumulateNew_cache_init_second_kernel :289-528);
 * then cache_assign_kernel gives bricks their slots and cache_fill_kernel
 * writes their voxels. */
__device__ __forceinline__ int tile_block_sum(int v, int *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int w = __reduce_add_sync(FULL, (unsigned)v);
    __syncthreads();
    if (lane == 0) red[wid] = w;
    __syncthreads();
    return red[0] + red[1];
}

template <bool VD>
__global__ void __launch_bounds__(64) cache_search_kernel(CacheBuildParams p)
{
    __shared__ int red[4];
    __shared__ int row_base;
    const int k = threadIdx.x, lane = k & 31, wid = k >> 5;
    const int n_alive_tiles = *p.n_alive_tiles;
    for (int ai = blockIdx.x; ai < n_alive_tiles; ai += gridDim.x) {
        __syncthreads();
        const int tile = p.alive_list[ai];
        CacheRay cr = p.rays[(size_t)tile * 64 + k];
        int bstep = p.block_step[tile];
        uint32_t mask = 0;
        bool found = false;
        /* one block-wide vote per depth brick (__syncthreads_or): any ray alive, any sample occupied */
        for (int guard = 0; guard < p.max_search; ++guard) {
            if (!__syncthreads_or(cr.alive)) break;
            if (bstep >= p.bZ) { cr.alive = 0; break; } /* beyond the frustum depth: stop the tile */
            float t1 = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
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
            if (__syncthreads_or(mask != 0u)) { found = true; break; }
            ++bstep;
            if (guard == p.max_search - 1) atomicOr(p.guard, 4);
        }
        const int total = found ? tile_block_sum(__popc(mask), red) : 0; /* found is block-uniform */
        const int n_alive = tile_block_sum(cr.alive, red);
        const bool processed = total > 0 && n_alive > 0;
        if (k == 0) {
            p.tile_n_samples[ai] = total;
            p.tile_processed[ai] = processed;
            p.tile_alive[tile] = n_alive > 0;
            p.block_step[tile] = bstep;
        }
        p.rays[(size_t)tile * 64 + k] = cr;
        if (!processed) continue;
        /* append the brick's samples to the iteration's rows, in (ray, step) order */
        const int cnt = __popc(mask);
        int incl = cnt;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, off);
            if (lane >= off) incl += v;
        }
        if (lane == 31) red[2 + wid] = incl;
        if (k == 0) row_base = atomicAdd(p.build_row_counter, total);
        __syncthreads();
        int row = row_base + incl - cnt + (wid ? red[2] : 0);
        int *rof = p.build_row_of + (size_t)ai * 512;
        float t1 = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const float t0 = t1;
            const float dt = calc_step(p.steps, t0);
            t1 = F_ADD(t0, dt);
            const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
            if ((mask >> s) & 1u) {
                const float3 cp = contract(p.scene, at(cr.o, cr.d, tm));
                p.build_rows[row] = make_float4(cp.x, cp.y, cp.z, 0.f);
                if (VD) /* the build's network input direction (src/cache_renderer.cu:1026) */
                    p.build_dirs[row] = make_float4((cr.d.x + 1.0f) / 2.0f, (cr.d.y + 1.0f) / 2.0f, (cr.d.z + 1.0f) / 2.0f, 0.f);
                rof[s * 64 + k] = row++;
            } else {
                rof[s * 64 + k] = -1;
            }
        }
    }
}

/* density network on every row of the iteration: log-density and the 8
 * latents (fp16, as NerfNetwork::inferenceLatents stores them); VD: the view-dependent network's first head on the rows' ray
 * directions */
template <bool VD>
__global__ void __launch_bounds__(128) cache_density_kernel(CacheBuildParams p)
{
    __shared__ uint2 Wsm[W_L3], Wfh[VD ? W_L3 : 1];
    __shared__ __align__(16) __half tiles[4][32 * TILE_STRIDE];
    for (int i = threadIdx.x; i < W_L3; i += blockDim.x) Wsm[i] = p.weights[i];
    if (VD)
        for (int i = threadIdx.x; i < W_L3; i += blockDim.x) Wfh[i] = p.weights_fh[i];
    __syncthreads();
    const int n = *p.build_row_counter;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __half *tile = tiles[w];
    __half *trow = tile + lane * TILE_STRIDE;
    const int lo = p.latent_offset;
    for (int b = blockIdx.x * 4 + w; b < (n + 31) / 32; b += gridDim.x * 4) {
        const int r = b * 32 + lane;
        if (r < n) {
            const float4 rw = p.build_rows[r];
            hash_encode(p.grid, p.table, make_float3(rw.x, rw.y, rw.z), reinterpret_cast<__half2 *>(trow));
        } else {
            for (int c = 0; c < 16; ++c) reinterpret_cast<uint32_t *>(trow)[c] = 0u;
        }
        __syncwarp();
        density_mlp(tile, Wsm, lane);
        __half logd = trow[16];
        if (VD) {
            /* the first head (NerfNetwork::inferenceLatents, include/nerf_network.h:183-197) on
             * [density outputs | SH of the build ray's direction]; its outputs take rows 1.. of the
             * head input (row 0 keeps the log-density) */
            uint4 o0 = reinterpret_cast<const uint4 *>(trow + 16)[0], o1 = reinterpret_cast<const uint4 *>(trow + 16)[1];
            __half2 sh[8];
            if (r < n) {
                float3 d01;
                if (p.build_dirs) {
                    const float4 d = p.build_dirs[r];
                    d01 = make_float3(d.x, d.y, d.z);
                } else { /* the per-ray fill: the row's ray (src/cache_renderer.cu:899) */
                    const float4 d = p.dir_states[p.dir_slot[r]].dt;
                    d01 = make_float3((d.x + 1.0f) / 2.0f, (d.y + 1.0f) / 2.0f, (d.z + 1.0f) / 2.0f);
                }
                sh16(d01, sh);
            } else {
                for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
            }
            __syncwarp();
            reinterpret_cast<uint4 *>(trow)[0] = o0;
            reinterpret_cast<uint4 *>(trow)[1] = o1;
            reinterpret_cast<uint4 *>(trow)[2] = *reinterpret_cast<const uint4 *>(sh);
            reinterpret_cast<uint4 *>(trow)[3] = *reinterpret_cast<const uint4 *>(sh + 4);
            __syncwarp();
            density_mlp(tile, Wfh, lane); /* the same 32 -> 64 -> 16 shape */
            /* rows 1..16 <- first-head outputs 0..15 */
            __syncwarp();
            for (int j = 15; j >= 1; --j) trow[16 + j] = trow[16 + j - 1];
            trow[16] = logd;
        }
        if (r < n) {
            p.build_den[r] = trow[16];
            uint32_t lw[4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                lw[q] = (uint32_t)__half_as_ushort(trow[16 + lo + 2 * q]) | ((uint32_t)__half_as_ushort(trow[17 + lo + 2 * q]) << 16);
            p.build_lat[r] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        __syncwarp();
    }
}

cudaError_t launch_cache_search(const CacheBuildParams &p, int grid, cudaStream_t s)
{
    if (p.view_dependent) cache_search_kernel<true><<<grid, 64, 0, s>>>(p);
    else cache_search_kernel<false><<<grid, 64, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_cache_density(const CacheBuildParams &p, int grid, cudaStream_t s)
{
    if (p.view_dependent) cache_density_kernel<true><<<grid, 128, 0, s>>>(p);
    else cache_density_kernel<false><<<grid, 128, 0, s>>>(p);
    return cudaGetLastError();
}

/* One warp per processed tile, rays lane and lane + 32 per lane:
 * density-only compositing over the brick's 8 steps
 * (accumulateNew_cache_init_second_kernel :349-393) and whether the brick
 * needs a slot (a visible sample). */
__global__ void __launch_bounds__(128) cache_composite_kernel(CacheBuildParams p)
{
    const int lane = threadIdx.x & 31;
    const int n_alive_tiles = *p.n_alive_tiles;
    const int n_warps = gridDim.x * (blockDim.x >> 5);
    for (int ai = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ai < n_alive_tiles; ai += n_warps) {
        if (!p.tile_processed[ai]) continue; /* uniform over the warp */
        const int tile = p.alive_list[ai];
        const int bstep = p.block_step[tile];
        const int *rof = p.build_row_of + (size_t)ai * 512;
        const float t1s = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
        int visible = 0, alive = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = h * 32 + lane;
            CacheRay cr = p.rays[(size_t)tile * 64 + k];
            float t1 = t1s;
            float T = cr.T;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const float t0 = t1;
                const float dt = calc_step(p.steps, t0);
                t1 = F_ADD(t0, dt);
                const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
                if (tm > cr.far_) { cr.alive = 0; continue; }
                const int row = rof[s * 64 + k];
                if (row < 0) continue;
                const float sigma = expf(__half2float(p.build_den[row]));
                const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-sigma * dt)));
                if (alpha > p.scene.alpha_thre) { T *= 1.0f - alpha; ++visible; }
                if (T < 1e-4f) cr.alive = 0;
            }
            cr.T = T;
            alive += cr.alive;
            p.rays[(size_t)tile * 64 + k] = cr;
        }
        const int n_visible = (int)__reduce_add_sync(FULL, (unsigned)visible);
        const int n_alive_post = (int)__reduce_add_sync(FULL, (unsigned)alive);
        if (lane == 0) {
            p.tile_need[ai] = n_visible > 0;
            p.tile_n_alive[ai] = n_alive_post;
        }
    }
}

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
 * has alive rays and did not overflow), emits the (tile, slot) fill jobs and
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

/* The 512 voxels of each brick that got a slot, written straight from the
 * iteration's network rows (zeros where the brick has no sample): density
 * slot and latent 0 per interpol_variant
 * (accumulateNew_cache_init_second_kernel :459-507).  Runs after
 * cache_assign_kernel, which advanced the tile's block step past the brick. */
__global__ void __launch_bounds__(256) cache_fill_kernel(CacheBuildParams p)
{
    __shared__ float s_dt[8];
    const int n_jobs = *p.n_jobs;
    const bool by_alpha = p.variant == VARIANT_ALPHA || p.variant == VARIANT_ALPHA_INTERMEDIATES;
    const bool lat0 = p.variant == VARIANT_DENSITY_INTERMEDIATES || p.variant == VARIANT_ALPHA_INTERMEDIATES;
    for (int j = blockIdx.x; j < n_jobs; j += gridDim.x) {
        const int ai = p.jobs[2 * j], slot = p.jobs[2 * j + 1];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int bstep = p.block_step[p.alive_list[ai]] - 1;
            float t1 = t_from_step(p.steps, F_ADD((float)(bstep * 8), p.steps.near_i));
            for (int s = 0; s < 8; ++s) {
                const float dt = calc_step(p.steps, t1);
                s_dt[s] = dt;
                t1 = F_ADD(t1, dt);
            }
        }
        __syncthreads();
        const int *rof = p.build_row_of + (size_t)ai * 512;
        Voxel *dst = reinterpret_cast<Voxel *>(p.voxels) + (size_t)slot * 512;
        for (int i = threadIdx.x; i < 512; i += blockDim.x) {
            const int row = rof[i];
            Voxel v;
            v.pad0 = v.pad1 = 0.f;
            if (row >= 0) {
                const float sigma = expf(__half2float(p.build_den[row]));
                const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-sigma * s_dt[i >> 6])));
                v.density = p.variant == VARIANT_INTERMEDIATES ? 0.f : by_alpha ? alpha : sigma; /* Intermediates: slot unwritten */
                v.isset = 1.0f;
                v.lat = p.build_lat[row];
                if (lat0) v.lat.x = (v.lat.x & 0xffff0000u) | (uint32_t)__half_as_ushort(__float2half_rn(v.density));
            } else {
                v.density = 0.f;
                v.isset = 0.f;
                v.lat = make_uint4(0, 0, 0, 0);
            }
            __stcs(reinterpret_cast<float4 *>(dst + i), make_float4(v.density, v.isset, 0.f, 0.f));
            __stcs(reinterpret_cast<uint4 *>(dst + i) + 1, v.lat);
        }
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

/* ------------------------------------------------------------------------- */
/* per-ray cache fill (CacheRenderer::initCache, src/cache_renderer.cu:571-928) */
/* ------------------------------------------------------------------------- */
/* known_ranges_to starts at StepsizeInfo::far, the RayPayload
 * termination_depth of rays that end neither by opacity nor by overflow
 * (initRayPayloads_common_kernel, src/renderer.cu:62-78) */
__global__ void pr_known_init_kernel(PerRayFillParams p)
{
    const int n = p.W * p.H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p.known_ranges[i] = p.steps.far_;
}

/* the froxel brick of a sample of pixel id at the midpoint tm, or -1 past the
 * frustum depth (bin = floor(step_from_t(t_mid) - near_i), :598-604) */
__device__ __forceinline__ int pr_brick(const PerRayFillParams &p, int id, float tm, int &bin)
{
    bin = (int)floorf(F_SUB(step_from_t(p.steps, tm), p.steps.near_i));
    const int bz = bin >> 3;
    if (bin < 0 || bz >= p.bZ) return -1;
    const int x = id % p.W, y = id / p.W;
    return (bz * p.bY + (y >> 3)) * p.bX + (x >> 3);
}

/* accumulate_cache_init_first_kernel (:571-623): per alive ray, the bricks of
 * its visible samples of this sub-iteration, until the transmittance falls
 * below 1e-4 (unclamped density) */
__global__ void __launch_bounds__(128) pr_mark_kernel(PerRayFillParams p, int it)
{
    const int n_alive = p.counters[it & 1];
    const RayState *states = p.states[it & 1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_alive; i += gridDim.x * blockDim.x) {
        const int2 rr = p.ray_rows[i];
        const int id = states[i].cnt.x;
        float T = states[i].acc.w;
        for (int k = 0; k < rr.y; ++k) {
            const int row = rr.x + k;
            const float density = expf(__half2float(p.den[row]));
            const float t0 = p.row_t0[row];
            const float dt = calc_step(p.steps, t0);
            const float t1 = F_ADD(t0, dt);
            const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
            const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-density * dt)));
            if (alpha > p.scene.alpha_thre) {
                T *= 1.0f - alpha;
                int bin;
                const int b = pr_brick(p, id, tm, bin);
                if (b < 0) break; /* beyond the frustum depth: pr_write ends the ray here */
                p.flag[b] = 1;
            }
            if (T < 1e-4f) break;
        }
    }
}

/* reserveNewBricks_kernel (:775-805) made deterministic: per brick column,
 * the number of bricks marked in this sub-iteration that hold no slot yet */
__global__ void __launch_bounds__(256) pr_count_kernel(PerRayFillParams p)
{
    const int n_cols = p.bX * p.bY;
    const size_t plane = (size_t)n_cols;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cols; c += gridDim.x * blockDim.x) {
        int n = 0;
        for (int z = 0; z < p.bZ; ++z) {
            const size_t b = (size_t)z * plane + c;
            n += p.flag[b] && !p.set[b];
        }
        p.col_count[c] = n;
    }
}

/* exclusive scan of the column counts from the slot counter (one CTA of 1024) */
__global__ void __launch_bounds__(1024) pr_scan_kernel(PerRayFillParams p)
{
    __shared__ int s_w[33];
    __shared__ int s_carry;
    const int n_cols = p.bX * p.bY;
    if (threadIdx.x == 0) {
        s_carry = p.slot_counter[0];
        p.slot_counter[1] = s_carry;
    }
    __syncthreads();
    for (int c0 = 0; c0 < n_cols; c0 += 1024) {
        const int c = c0 + threadIdx.x;
        const int v = c < n_cols ? p.col_count[c] : 0;
        int total;
        const int ex = block_exclusive_scan(v, total, s_w);
        if (c < n_cols) p.col_base[c] = s_carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) p.slot_counter[0] = s_carry;
}

/* slots in (column, depth) order; a slot beyond the capacity leaves the brick
 * without one (packed index -1), as the reference's overflow does; clears the
 * marks for the next sub-iteration */
__global__ void __launch_bounds__(256) pr_reserve_kernel(PerRayFillParams p)
{
    const int n_cols = p.bX * p.bY;
    const size_t plane = (size_t)n_cols;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cols; c += gridDim.x * blockDim.x) {
        int slot = p.col_base[c];
        for (int z = 0; z < p.bZ; ++z) {
            const size_t b = (size_t)z * plane + c;
            if (!p.flag[b]) continue;
            p.flag[b] = 0;
            if (p.set[b]) continue;
            const bool overflow = slot >= p.capacity;
            if (!overflow) {
                const int sx = slot / (p.dY * p.dZ), sy = (slot - sx * p.dY * p.dZ) / p.dZ;
                const int sz = slot - sx * p.dY * p.dZ - sy * p.dZ;
                p.packed_index[b] = (sx << 20) | (sy << 10) | sz;
                p.set[b] = 1;
            } else {
                p.packed_index[b] = -1;
            }
            ++slot;
        }
    }
}

/* the slots reserved in this sub-iteration start out empty (Cache::
 * setDataArraysZero, src/cache_renderer.cu:854) */
__global__ void __launch_bounds__(256) pr_zero_kernel(PerRayFillParams p)
{
    const int s0 = min(p.slot_counter[1], p.capacity), s1 = min(p.slot_counter[0], p.capacity);
    uint4 *v = reinterpret_cast<uint4 *>(p.voxels);
    const size_t n = (size_t)(s1 - s0) * 1024;
    const size_t base = (size_t)s0 * 1024;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        v[base + i] = make_uint4(0, 0, 0, 0);
}

/* accumulate_cache_init_second_kernel (:625-773): per alive ray, the voxels of
 * its visible samples (density clamped to exp(10)), the density slot and
 * latent 0 per interpol_variant; a sample whose brick got no slot (or lies
 * beyond the frustum depth) ends the ray at its t0, transmittance below 1e-4
 * at its t1.  Rays that end write their termination depth to known_ranges_to
 * (writeImageBuffer_cache_init_kernel, :807-827); the others are compacted
 * into the next alive list. */
__global__ void __launch_bounds__(128) pr_write_kernel(PerRayFillParams p, int it)
{
    const int n_alive = p.counters[it & 1];
    RayState *states = p.states[it & 1];
    RayState *next = p.states[(it + 1) & 1];
    const bool by_alpha = p.variant == VARIANT_ALPHA || p.variant == VARIANT_ALPHA_INTERMEDIATES;
    const bool lat0 = p.variant == VARIANT_DENSITY_INTERMEDIATES || p.variant == VARIANT_ALPHA_INTERMEDIATES;
    Voxel *vox = reinterpret_cast<Voxel *>(p.voxels);
    for (int base = blockIdx.x * blockDim.x; base < n_alive; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        bool alive = false;
        RayState st;
        if (i < n_alive) {
            st = states[i];
            const int2 rr = p.ray_rows[i];
            const int id = st.cnt.x;
            float T = st.acc.w, term = p.steps.far_;
            alive = st.cnt2.y == 0; /* the march ended the ray past its far bound */
            for (int k = 0; k < rr.y; ++k) {
                const int row = rr.x + k;
                const float density = expf(fminf(__half2float(p.den[row]), 10.0f));
                const float t0 = p.row_t0[row];
                const float dt = calc_step(p.steps, t0);
                const float t1 = F_ADD(t0, dt);
                const float tm = F_MUL(F_ADD(t0, t1), 0.5f);
                const float alpha = fminf(1.0f, fmaxf(0.0f, 1.0f - expf(-density * dt)));
                if (alpha > p.scene.alpha_thre) {
                    T *= 1.0f - alpha;
                    int bin;
                    const int b = pr_brick(p, id, tm, bin);
                    const int packed = b >= 0 ? p.packed_index[b] : -1;
                    if (packed < 0) { /* no slot: the cache overflowed here */
                        alive = false;
                        term = t0;
                        break;
                    }
                    const int x = id % p.W, y = id / p.W;
                    const int slot = ((packed >> 20) & 1023) * (p.dY * p.dZ) + ((packed >> 10) & 1023) * p.dZ + (packed & 1023);
                    Voxel v;
                    v.density = p.variant == VARIANT_INTERMEDIATES ? 0.f : by_alpha ? alpha : density;
                    v.isset = 1.0f;
                    v.pad0 = v.pad1 = 0.f;
                    v.lat = p.lat[row];
                    if (lat0) v.lat.x = (v.lat.x & 0xffff0000u) | (uint32_t)__half_as_ushort(__float2half_rn(v.density));
                    vox[(size_t)slot * 512 + (bin & 7) * 64 + (y & 7) * 8 + (x & 7)] = v;
                }
                if (T < 1e-4f) {
                    alive = false;
                    term = t1;
                    break;
                }
            }
            st.acc.w = T;
            if (!alive) p.known_ranges[id] = term;
        }
        const unsigned m = __ballot_sync(0xffffffffu, alive);
        int wbase = 0;
        if ((threadIdx.x & 31) == 0 && m) wbase = atomicAdd(p.counters + ((it + 1) & 1), __popc(m));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        if (alive) {
            unsigned lt;
            asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
            next[wbase + __popc(m & lt)] = st;
        }
    }
}

}  // namespace fvc
