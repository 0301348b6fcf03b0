/*
 * fvc_backward.cu - adjoint of the plain render: loss, network backward with
 * hash-table scatter, gradient read-out.
 *
 * The reference has no backward pass; this is the differentiable form of its
 * plain renderer (PerformanceRenderer::render, src/performance_renderer.cu:
 * 214-286).  The loss is the mean over rays of the squared error of the
 * white-background pixel (C + T, writeImageBuffer_performance_kernel,
 * src/performance_renderer.cu:127-149).
 *
 * Two forms of the network backward:
 *   - wf_net_bwd_tc_kernel (the default) runs on the tcgen05 tensor cores,
 *     warp-specialised, 128 rows per tile, with the weight gradients
 *     accumulated in TMEM (its comment block below has the layout);
 *   - wf_net_bwd_kernel (the mma.sync network path) takes one warp per 32
 *     rows (mma.sync m16n8k16, fp16 or bf16 operands like the forward MLP,
 *     fp32 accumulation).
 * Both recompute the forward activations of the rows (hash features, density
 * hidden layer, head input [latents | SH | 1-padding], head hidden layers)
 * into shared memory; the gradient tile then walks back through the layers.
 * In the mma.sync form:  Input gradients are tile x weight-pack products;
 * weight gradients dW = G^T X take both operands from the shared tiles with
 * ldmatrix.trans and accumulate in a per-CTA fp32 copy of the parameter
 * blobs, added to the global gradients once per launch.  Feature gradients
 * scatter into the fp32 table gradient with red.global.add.v2.f32, weighted by
 * the trilinear weights of the forward.
 *
 * Gradients carry a loss scale (per-ray dL/dC = 2 e * scale) so that fp16
 * gradient tiles stay in the normal range; the read-out kernel divides it
 * out together with the 1/N of the mean.
 */
#include <algorithm>
#include <cstddef>

#include <cuda_bf16.h>

#include "fvc_kernels.h"

namespace fvc {

constexpr unsigned FULLMASK = 0xffffffffu;
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

/* the 16-bit element type of the MLP: fp16 (PREC 0) or bf16 (PREC 1); tiles
 * hold raw 16-bit values */
template <int PREC> struct E16;
template <> struct E16<0> {
    static __device__ __forceinline__ uint32_t pack(float a, float b) { return pack_h2(a, b); }
    static __device__ __forceinline__ float2 unpack(uint32_t v) { return __half22float2(*reinterpret_cast<__half2 *>(&v)); }
    static __device__ __forceinline__ uint16_t one(float v) { return __half_as_ushort(__float2half_rn(v)); }
    static __device__ __forceinline__ float flt(uint16_t v) { return __half2float(__ushort_as_half(v)); }
    static __device__ __forceinline__ void mma(float (&c)[4], const uint32_t (&a)[4], uint2 b) { mma16816(c, a, b); }
};
template <> struct E16<1> {
    static __device__ __forceinline__ uint32_t pack(float a, float b)
    {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    static __device__ __forceinline__ float2 unpack(uint32_t v) { return __bfloat1622float2(*reinterpret_cast<__nv_bfloat162 *>(&v)); }
    static __device__ __forceinline__ uint16_t one(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
    static __device__ __forceinline__ float flt(uint16_t v) { return __bfloat162float(__ushort_as_bfloat16(v)); }
    static __device__ __forceinline__ void mma(float (&c)[4], const uint32_t (&a)[4], uint2 b)
    {
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                     : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
    }
};

constexpr int BW_WARPS = 8; /* 8 x 23.5 KB of row tiles + 40 KB of dW: one CTA of 8 warps per SM */
constexpr int S32 = 40;  /* tile strides in halfs: 80 B and 144 B rows, 16-byte aligned for ldmatrix */
constexpr int S64 = 72;
constexpr int DF_STRIDE = 36; /* fp32 feature-gradient rows (aliases the A3 tile) */
constexpr int DW_FLOATS = GB_BASE + 64 * 32 + 64 * 64 + 16 * 64;

struct __align__(16) BwdWarp {
    uint16_t F[32 * S32];   /* hash features */
    uint16_t H1[32 * S64];  /* density hidden layer (ReLU) */
    uint16_t IN[32 * S32];  /* head input: latents 0..7, SH 8..23, 1.0 at 24..31 */
    uint16_t A3[32 * S64];  /* head hidden 1; later the fp32 feature gradients */
    uint16_t A4[32 * S64];  /* head hidden 2 */
    uint16_t G[32 * S64];   /* the gradient tile walking back */
};

struct __align__(16) BwdSmem {
    float dW[DW_FLOATS];  /* base blob, then head blob */
    BwdWarp w[BW_WARPS];
};

__device__ __forceinline__ void lda_tile(const uint16_t *t, int stride, int m0, int k0, int lane, uint32_t (&a)[4])
{
    const int g = lane >> 2, q = lane & 3;
    const uint16_t *r0 = t + (m0 + g) * stride + k0 + 2 * q;
    const uint16_t *r1 = r0 + 8 * stride;
    a[0] = *reinterpret_cast<const uint32_t *>(r0);
    a[1] = *reinterpret_cast<const uint32_t *>(r1);
    a[2] = *reinterpret_cast<const uint32_t *>(r0 + 8);
    a[3] = *reinterpret_cast<const uint32_t *>(r1 + 8);
}

/* c[32 x N] = A[32 x K] (shared tile) * B (fragment pack, N/8 n-tiles x K/16 k-steps) */
template <int PREC, int K, int N>
__device__ __forceinline__ void warp_mm(const uint16_t *A, int sa, const uint2 *__restrict__ Bp, int lane, float (&c)[2][N / 8][4])
{
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int j = 0; j < N / 8; ++j) c[m][j][0] = c[m][j][1] = c[m][j][2] = c[m][j][3] = 0.f;
#pragma unroll
    for (int s = 0; s < K / 16; ++s) {
        uint32_t a0[4], a1[4];
        lda_tile(A, sa, 0, 16 * s, lane, a0);
        lda_tile(A, sa, 16, 16 * s, lane, a1);
#pragma unroll
        for (int j = 0; j < N / 8; ++j) {
            const uint2 b = __ldg(&Bp[(j * (K / 16) + s) * 32 + lane]);
            E16<PREC>::mma(c[0][j], a0, b);
            E16<PREC>::mma(c[1][j], a1, b);
        }
    }
}

__device__ __forceinline__ float clamp_h(float v) { return fminf(fmaxf(v, -65000.f), 65000.f); }

/* c -> fp16 tile; mode 0 as is, 1 ReLU, 2 zero where the mask tile is not > 0 */
template <int PREC, int N>
__device__ __forceinline__ void st_tile(uint16_t *T, int st, const float (&c)[2][N / 8][4], int lane, int mode,
                                        const uint16_t *M = nullptr, int sm = 0)
{
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int j = 0; j < N / 8; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = 16 * m + g + 8 * h, col = 8 * j + 2 * q;
                float v0 = c[m][j][2 * h], v1 = c[m][j][2 * h + 1];
                if (mode == 1) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                if (mode == 2) {
                    const float2 mk = E16<PREC>::unpack(*reinterpret_cast<const uint32_t *>(M + row * sm + col));
                    if (!(mk.x > 0.f)) v0 = 0.f;
                    if (!(mk.y > 0.f)) v1 = 0.f;
                }
                *reinterpret_cast<uint32_t *>(T + row * st + col) = E16<PREC>::pack(clamp_h(v0), clamp_h(v1));
            }
}

__device__ __forceinline__ void ldsm4t(uint32_t (&r)[4], const uint16_t *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

/* the shared dW copy keeps row-major rows of I floats with the column
 * XOR-swizzled by 4 * (row % 8): the 32 lanes of an accumulator fragment
 * (rows g, columns 2q) then fall into 16 banks instead of 4 */
__device__ __forceinline__ int dw_col(int row, int col) { return col ^ ((row & 7) << 2); }

/* dW (O x I, row-major fp32, shared, swizzled) += G^T X over the warp's 32
 * rows; G: 32 x O, X: 32 x I, both fp16 shared tiles. */
template <int PREC, int O, int I>
__device__ __forceinline__ void warp_dw(const uint16_t *G, int sg, const uint16_t *X, int sx, float *dW, int lane)
{
    const int g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int mt = 0; mt < O / 16; ++mt) {
        uint32_t a[2][4];
#pragma unroll
        for (int s = 0; s < 2; ++s)
            ldsm4t(a[s], G + (16 * s + (lane & 7) + ((lane >> 4) << 3)) * sg + 16 * mt + ((lane >> 3) & 1) * 8);
#pragma unroll
        for (int nt = 0; nt < I / 8; nt += 2) {
            float d[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                uint32_t b[4];
                ldsm4t(b, X + (16 * s + (lane & 7) + ((lane >> 3) & 1) * 8) * sx + 8 * (nt + (lane >> 4)));
                E16<PREC>::mma(d[0], a[s], make_uint2(b[0], b[1]));
                E16<PREC>::mma(d[1], a[s], make_uint2(b[2], b[3]));
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r0 = 16 * mt + g, r1 = r0 + 8, c = 8 * (nt + h) + 2 * q;
                atomicAdd(dW + r0 * I + dw_col(r0, c), d[h][0]);
                atomicAdd(dW + r0 * I + dw_col(r0, c + 1), d[h][1]);
                atomicAdd(dW + r1 * I + dw_col(r1, c), d[h][2]);
                atomicAdd(dW + r1 * I + dw_col(r1, c + 1), d[h][3]);
            }
        }
    }
}

__device__ __forceinline__ void red_add2(float *a, float x, float y)
{
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};\n" ::"l"(a), "f"(x), "f"(y) : "memory");
}

/* adjoint of hash_encode: corner indices and trilinear weights as the forward */
__device__ __forceinline__ void hash_scatter(const DevGrid &g, float *gt, float3 pos, const float *dF)
{
    for (int l = 0; l < g.n_levels; ++l) {
        const float fx0 = dF[2 * l], fy0 = dF[2 * l + 1];
        if (fx0 == 0.f && fy0 == 0.f) continue;
        const float sc = g.scale[l];
        const float px = __fmaf_rn(sc, pos.x, 0.5f), py = __fmaf_rn(sc, pos.y, 0.5f), pz = __fmaf_rn(sc, pos.z, 0.5f);
        const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
        const uint32_t gx = (uint32_t)(int)fx, gy = (uint32_t)(int)fy, gz = (uint32_t)(int)fz;
        const float wx = __fsub_rn(px, fx), wy = __fsub_rn(py, fy), wz = __fsub_rn(pz, fz);
        const uint32_t size = g.size[l];
        float *tl = gt + 2 * (size_t)g.offset[l];
        const bool dense = (g.dense_mask >> l) & 1u;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const uint32_t cx = gx + (c & 1), cy = gy + ((c >> 1) & 1), cz = gz + ((c >> 2) & 1);
            uint32_t i;
            if (dense) {
                i = cx + cy * g.res[l] + cz * g.res2[l];
                if (i >= size) i -= size;
            } else {
                i = (cx ^ (cy * 2654435761u) ^ (cz * 805459861u)) & (size - 1u);
            }
            const float w = ((c & 1) ? wx : 1.0f - wx) * ((c & 2) ? wy : 1.0f - wy) * ((c & 4) ? wz : 1.0f - wz);
            red_add2(tl + 2 * (size_t)i, w * fx0, w * fy0);
        }
    }
}

__device__ __forceinline__ float3 row_dir01(const RayState *states, int slot)
{
    const float4 d = states[slot].dt;
    return make_float3((d.x + 1.0f) / 2.0f, (d.y + 1.0f) / 2.0f, (d.z + 1.0f) / 2.0f);
}

template <int PREC, int HH>
__global__ void __launch_bounds__(BW_WARPS * 32, 1) wf_net_bwd_kernel(RenderParams p, BwdParams b, int it)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BwdSmem &S = *reinterpret_cast<BwdSmem *>(smem_raw);
    const int n_rows = p.counters[6];
    if (n_rows == 0) return;
    for (int i = threadIdx.x; i < DW_FLOATS; i += blockDim.x) S.dW[i] = 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = lane_id();
    BwdWarp &W = S.w[warp];
    float *dWb = S.dW, *dWh = S.dW + GB_BASE;
    const RayState *states = p.states[it & 1];
    const int lo = p.latent_offset;
    const int n_tiles = (n_rows + 31) / 32;
    uint16_t *inr = W.IN + lane * S32;
    uint16_t *gr = W.G + lane * S64;
    using T16 = E16<PREC>;
    for (int tile = blockIdx.x * BW_WARPS + warp; tile < n_tiles; tile += gridDim.x * BW_WARPS) {
        const int k = tile * 32 + lane;
        const int r = k < n_rows ? p.grad_res_list[k] : -1;
        float4 dout = make_float4(0.f, 0.f, 0.f, 0.f);
        float3 pos = make_float3(0.f, 0.f, 0.f);
        __half2 sh[8];
        if (r >= 0) {
            dout = p.row_dout[r];
            const float4 pw = p.row_pay[r];
            pos = make_float3(pw.x, pw.y, pw.z);
            sh16(row_dir01(states, p.row_slot[r]), sh);
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
        }
        /* ---- forward recomputation ---- */
        __half2 feat[16];
        hash_encode<4>(p.grid, p.table, pos, feat);
        uint32_t *fr = reinterpret_cast<uint32_t *>(W.F + lane * S32);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const float2 f = __half22float2(feat[q]);
            fr[q] = PREC == 0 ? *reinterpret_cast<const uint32_t *>(&feat[q]) : T16::pack(f.x, f.y);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float2 f = __half22float2(sh[q]);
            reinterpret_cast<uint32_t *>(inr + 8)[q] = PREC == 0 ? *reinterpret_cast<const uint32_t *>(&sh[q]) : T16::pack(f.x, f.y);
        }
#pragma unroll
        for (int q = 24; q < 32; ++q) inr[q] = T16::one(1.0f);
        __syncwarp();
        {
            float c[2][8][4];
            warp_mm<PREC, 32, 64>(W.F, S32, b.w + BW_F1, lane, c);
            st_tile<PREC, 64>(W.H1, S64, c, lane, 1);
        }
        __syncwarp();
        {
            float c[2][2][4];
            warp_mm<PREC, 64, 16>(W.H1, S64, b.w + BW_F2, lane, c);
            st_tile<PREC, 16>(W.G, S64, c, lane, 0);
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 8; ++q) inr[q] = gr[lo + q];
        __syncwarp();
        {
            float c[2][8][4];
            warp_mm<PREC, 32, 64>(W.IN, S32, b.w + BW_F3, lane, c);
            st_tile<PREC, 64>(W.A3, S64, c, lane, 1);
        }
        __syncwarp();
        const uint16_t *last = W.A3;
        if (HH == 2) {
            float c[2][8][4];
            warp_mm<PREC, 64, 64>(W.A3, S64, b.w + BW_F4, lane, c);
            st_tile<PREC, 64>(W.A4, S64, c, lane, 1);
            __syncwarp();
            last = W.A4;
        }
        /* ---- backward: output layer ---- */
        gr[0] = T16::one(clamp_h(dout.x));
        gr[1] = T16::one(clamp_h(dout.y));
        gr[2] = T16::one(clamp_h(dout.z));
#pragma unroll
        for (int q = 3; q < 16; ++q) gr[q] = 0;
        __syncwarp();
        warp_dw<PREC, 16, 64>(W.G, S64, last, S64, dWh + b.head_w5, lane);
        {
            float c[2][8][4];
            warp_mm<PREC, 16, 64>(W.G, S64, b.w + BW_B5, lane, c);
            __syncwarp();
            st_tile<PREC, 64>(W.G, S64, c, lane, 2, last, S64);
        }
        __syncwarp();
        if (HH == 2) {
            warp_dw<PREC, 64, 64>(W.G, S64, W.A3, S64, dWh + GH_W4, lane);
            float c[2][8][4];
            warp_mm<PREC, 64, 64>(W.G, S64, b.w + BW_B4, lane, c);
            __syncwarp();
            st_tile<PREC, 64>(W.G, S64, c, lane, 2, W.A3, S64);
            __syncwarp();
        }
        /* ---- head layer 1: G = dA3 ---- */
        warp_dw<PREC, 64, 32>(W.G, S64, W.IN, S32, dWh + GH_W3, lane);
        float dl[2][1][4];
        warp_mm<PREC, 64, 8>(W.G, S64, b.w + BW_B3, lane, dl); /* d latents = head-input cols 0..7 */
        __syncwarp();
        /* ---- density network: G = d(out2) ---- */
#pragma unroll
        for (int q = 0; q < 16; ++q) gr[q] = 0;
        __syncwarp();
        {
            const int g = lane >> 2, q = lane & 3;
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint16_t *d = W.G + (16 * m + g + 8 * h) * S64 + lo + 2 * q;
                    d[0] = T16::one(clamp_h(dl[m][0][2 * h]));
                    d[1] = T16::one(clamp_h(dl[m][0][2 * h + 1]));
                }
        }
        __syncwarp();
        gr[0] = T16::one(clamp_h(T16::flt(gr[0]) + dout.w));
        __syncwarp();
        warp_dw<PREC, 16, 64>(W.G, S64, W.H1, S64, dWb + GB_W2, lane);
        {
            float c[2][8][4];
            warp_mm<PREC, 16, 64>(W.G, S64, b.w + BW_B2, lane, c);
            __syncwarp();
            st_tile<PREC, 64>(W.G, S64, c, lane, 2, W.H1, S64);
        }
        __syncwarp();
        warp_dw<PREC, 64, 32>(W.G, S64, W.F, S32, dWb + GB_W1, lane);
        float *dF = reinterpret_cast<float *>(W.A3);
        {
            float c[2][4][4];
            warp_mm<PREC, 64, 32>(W.G, S64, b.w + BW_B1, lane, c);
            const int g = lane >> 2, q = lane & 3;
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        float *d = dF + (16 * m + g + 8 * h) * DF_STRIDE + 8 * j + 2 * q;
                        d[0] = c[m][j][2 * h];
                        d[1] = c[m][j][2 * h + 1];
                    }
        }
        __syncwarp();
        if (r >= 0) hash_scatter(p.grid, b.g_table, pos, dF + lane * DF_STRIDE);
        __syncwarp();
    }
    __syncthreads();
    /* un-swizzle each layer's rows while adding to the global gradients */
    auto flush = [&](const float *src, float *dst, int n, int I) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int row = i / I, col = i - row * I;
            const float v = src[row * I + dw_col(row, col)];
            if (v != 0.f) atomicAdd(dst + i, v);
        }
    };
    flush(dWb + GB_W1, b.g_base + GB_W1, 64 * 32, 32);
    flush(dWb + GB_W2, b.g_base + GB_W2, 16 * 64, 64);
    flush(dWh + GH_W3, b.g_head + GH_W3, 64 * 32, 32);
    if (HH == 2) flush(dWh + GH_W4, b.g_head + GH_W4, 64 * 64, 64);
    flush(dWh + b.head_w5, b.g_head + b.head_w5, 16 * 64, 64);
}

/* ------------------------------------------------------------------------- */
/* network adjoint on the 5th-generation tensor cores                        */
/* ------------------------------------------------------------------------- */
/* Warp-specialised: two CTAs per SM, each CTA persistent over 128-row
 * tiles, 128 + 128 * FVC_BT_HASH_SPLIT threads.
 *   - MMA warps 0..3: thread t owns row t of a tile and TMEM lane t; thread 0
 *     issues the tcgen05 MMAs, the warps wait (bounded) and run the
 *     epilogues.  They synchronise among themselves with named barrier 1.
 *   - hash warps 4..: thread 128 + h fetches row h & 127 of the next tile,
 *     runs the hash encode of its share of the 16 levels into a
 *     double-buffered feature / head-input tile, and scatters that share of
 *     the feature gradients of the tile before, read from TMEM.  With the
 *     default split of 1 there are 4 hash warps, one thread per row.
 * The hash gathers and the table-gradient atomics (L2-bound) thus overlap the
 * MMA stage chain of another tile.  Handoffs use mbarriers:
 *   in_full[b]  hash -> MMA: F[b], IN[b] (SH, 1-padding) and dout[b] written;
 *   df_full     MMA -> hash: the tile's feature gradients sit in TMEM columns
 *               224..255 and its last MMAs (which read F[b], IN[b]) are done;
 *   df_empty    hash -> MMA: those columns have been read.
 * Each activation and gradient of a tile sits in its own canonical K-major
 * shared tile (8-row x 16-byte core matrices, see fvc_tc.cuh), so it serves
 * as the K-major A operand of the next layer (forward X W^T, input gradient
 * G W) and as an MN-major operand of the weight-gradient MMA dW = G^T X,
 * whose contraction runs over the tile's 128 rows.  Read MN-major, a tile of
 * C columns has its 8-column groups SBO = 128 bytes apart and its 8-row
 * groups LBO = C / 8 * 128 bytes apart.  The input-gradient MMAs read the
 * forward weight tiles MN-major as their B = W, so one copy of each weight
 * serves both directions.
 * The weight gradients accumulate in TMEM over every tile the CTA takes and
 * are added to the global blobs once per launch; no shared-memory atomics.
 * The weight-gradient MMAs use M = 128 with their 64 meaningful rows in TMEM
 * lanes 0..63: a 64-column tile read MN-major with M = 128 runs up to 1023
 * bytes past its end, which stays inside the next tile.
 * Gradient tiles reuse the activation tile whose mask they need, in place,
 * once the MMAs that read that tile have completed.
 * TMEM columns: 0..63 layer accumulator; 64..127 dW4; 128..159 dW3;
 * 160..191 dW1; 192..207 dW5^T; 208..223 dW2^T; 224..255 feature gradients. */
#ifndef FVC_BT_HASH_GROUP
#define FVC_BT_HASH_GROUP 4 /* hash levels whose gathers are in flight together */
#endif
constexpr int BT_COLS = 256;
constexpr int BT_D0 = 0, BT_DW4 = 64, BT_DW3 = 128, BT_DW1 = 160, BT_DW5T = 192, BT_DW2T = 208, BT_DF = 224;
constexpr long long BT_WAIT_LIMIT = 2000000000ll; /* ~1 s of SM clocks */
#ifndef FVC_BT_HASH_SPLIT
#define FVC_BT_HASH_SPLIT 1 /* hash threads per row (each takes 16 / split levels); 1 and 2 measured alike */
#endif
constexpr int BT_SPLIT = FVC_BT_HASH_SPLIT, BT_NL = 16 / BT_SPLIT;
constexpr int BT_HASH_THREADS = 128 * BT_SPLIT, BT_THREADS = 128 + BT_HASH_THREADS;
static_assert(BT_SPLIT == 1 || BT_SPLIT == 2, "1 or 2 hash threads per row");

struct __align__(128) BtSmem {
    uint8_t W[TB_BYTES];
    uint8_t H1[128 * 64 * 2];     /* density hidden layer, later its gradient */
    uint8_t A3[128 * 64 * 2];     /* head hidden 1, later its gradient */
    uint8_t A4[128 * 64 * 2];     /* head hidden 2, later its gradient */
    uint8_t F[2][128 * 32 * 2];   /* hash features */
    uint8_t IN[2][128 * 32 * 2];  /* head input [latents | SH | 1.0] */
    uint8_t G16[128 * 16 * 2];    /* output-layer gradient, later the density-network output gradient */
    float4 dout[2][128];          /* the rows' output gradients */
    uint64_t mbar, in_full[2], df_full, df_empty;
    uint32_t tmem_base;
};
static_assert(2 * (sizeof(BtSmem) + 1024) <= 228 * 1024, "two CTAs per SM");
static_assert(2 * BT_COLS <= 512, "two CTAs per SM in TMEM");
static_assert(offsetof(BtSmem, F) - offsetof(BtSmem, A4) == 128 * 64 * 2 && offsetof(BtSmem, A3) - offsetof(BtSmem, H1) == 128 * 64 * 2 &&
                  offsetof(BtSmem, A4) - offsetof(BtSmem, A3) == 128 * 64 * 2 && sizeof(BtSmem::F) >= 1024,
              "each 64-column tile read MN-major with M = 128 is followed by 1 KB of other tiles");

__device__ __forceinline__ void bt_st(uint8_t *tile, int row, int c, int K, uint4 v)
{
    *reinterpret_cast<uint4 *>(tile + kmajor_offset(row, 8 * c, K)) = v;
}
__device__ __forceinline__ uint4 bt_ld(const uint8_t *tile, int row, int c, int K)
{
    return *reinterpret_cast<const uint4 *>(tile + kmajor_offset(row, 8 * c, K));
}

/* D = A (128 x K, K-major tile) * B^T (N x K, K-major tile) */
__device__ __forceinline__ void bt_mma_k(uint32_t d, const uint8_t *a, const uint8_t *b, int K, int N, bool bf16)
{
    const uint32_t sbo = (uint32_t)(K / 8) * 128u, id = idesc_f16(128, N, bf16);
    const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
    for (int kc = 0; kc < K / 16; ++kc)
        tc_mma_f16(d, umma_desc(a0 + 256u * kc, 128u, sbo), umma_desc(b0 + 256u * kc, 128u, sbo), id, kc > 0 ? 1u : 0u);
}

/* D = A (128 x K, K-major tile) * W (K x N) where W is a weight tile stored
 * K-major for the forward (bw columns per row, row = the K index here), read
 * MN-major */
__device__ __forceinline__ void bt_mma_kw(uint32_t d, const uint8_t *a, const uint8_t *w, int bw, int K, int N, bool bf16)
{
    const uint32_t sbo = (uint32_t)(K / 8) * 128u, id = idesc_f16(128, N, bf16) | (1u << 16);
    const uint32_t lb = (uint32_t)(bw / 8) * 128u;
    const uint32_t a0 = smem_u32(a), b0 = smem_u32(w);
    for (int kc = 0; kc < K / 16; ++kc)
        tc_mma_f16(d, umma_desc(a0 + 256u * kc, 128u, sbo), umma_desc(b0 + 2u * lb * kc, lb, 128u), id, kc > 0 ? 1u : 0u);
}

/* D (+)= A^T B over the 128 tile rows: A a tile of ca columns (M = 128 read
 * from it), B a tile of N columns, both MN-major */
__device__ __forceinline__ void bt_mma_mn(uint32_t d, const uint8_t *a, int ca, const uint8_t *b, int N, bool bf16, bool acc)
{
    const uint32_t id = idesc_f16(128, N, bf16) | (1u << 15) | (1u << 16);
    const uint32_t la = (uint32_t)(ca / 8) * 128u, lb = (uint32_t)(N / 8) * 128u;
    const uint32_t a0 = smem_u32(a), b0 = smem_u32(b);
    for (int s = 0; s < 8; ++s)
        tc_mma_f16(d, umma_desc(a0 + 2u * la * s, la, 128u), umma_desc(b0 + 2u * lb * s, lb, 128u), id, (acc || s > 0) ? 1u : 0u);
}

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(mbar)) : "memory");
}

/* bounded wait on a phase parity; a phase that never completes clears ok */
__device__ __forceinline__ void bt_wait_on(uint64_t *mbar, uint32_t parity, bool &ok)
{
    if (ok && !mbar_wait(mbar, parity, BT_WAIT_LIMIT)) ok = false;
    tc_fence_after();
}

/* MMA warps: rewritten rows visible to the tensor core, TMEM reads ordered
 * before the next MMA; named barrier 1 over the 128 MMA-warp threads, OR of
 * the failure flags */
__device__ __forceinline__ bool bt_publish(bool ok)
{
    fence_proxy_async();
    tc_fence_before();
    uint32_t bad;
    asm volatile("{\n .reg .pred p, q;\n setp.eq.u32 p, %1, 0;\n bar.red.or.pred q, 1, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(bad)
                 : "r"(ok ? 1u : 0u)
                 : "memory");
    return bad == 0u;
}

/* 64 accumulator columns -> ReLU -> 16-bit row of a 64-column tile */
template <int PREC>
__device__ __forceinline__ void bt_epi_act(uint32_t taddr, uint8_t *dst, int row)
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float v[32];
        tmem_ld32(taddr + 32 * h, v);
        tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int c = 8 * q + 2 * i;
                w[i] = E16<PREC>::pack(clamp_h(fmaxf(v[c], 0.f)), clamp_h(fmaxf(v[c + 1], 0.f)));
            }
            bt_st(dst, row, 4 * h + q, 64, make_uint4(w[0], w[1], w[2], w[3]));
        }
    }
}

/* 64 accumulator columns, zeroed where the activation row is not > 0, written
 * over that activation row (64-column tile) */
template <int PREC>
__device__ __forceinline__ void bt_epi_grad(uint32_t taddr, uint8_t *tile, int row)
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float v[32];
        tmem_ld32(taddr + 32 * h, v);
        uint4 mk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) mk[q] = bt_ld(tile, row, 4 * h + q, 64);
        tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t m4[4] = {mk[q].x, mk[q].y, mk[q].z, mk[q].w};
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int c = 8 * q + 2 * i;
                const float2 m = E16<PREC>::unpack(m4[i]);
                const float a = m.x > 0.f ? v[c] : 0.f, b = m.y > 0.f ? v[c + 1] : 0.f;
                w[i] = E16<PREC>::pack(clamp_h(a), clamp_h(b));
            }
            bt_st(tile, row, 4 * h + q, 64, make_uint4(w[0], w[1], w[2], w[3]));
        }
    }
}

__device__ __forceinline__ void red_add4(float *a, float x, float y, float z, float w)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"l"(a), "f"(x), "f"(y), "f"(z), "f"(w) : "memory");
}

/* levels at which consecutive samples of a ray usually share a cell (cells
 * wider than about one step) */
constexpr int SC_PAIR_LEVELS = 10;

/* Adjoint of hash_encode over levels l0 .. l0 + NL - 1 of the 16-level grid,
 * called by all 32 lanes of a warp (rows without a gradient pass zeros).
 * Per level:
 *   - lanes 2j and 2j+1 in the same cell at a coarse level merge: the odd
 *     lane hands its trilinear weights and feature gradient to the even lane,
 *     which adds both rows' contributions to the 8 corners;
 *   - x-neighbour corners whose table entries form an aligned pair
 *     {2i, 2i+1} (a hashed level's cell with even x, or adjacent dense
 *     indices) go out as one 16-byte red.global.add.v4.f32.
 * The table receives the same sums with fewer L2 atomics. */
template <int NL>
__device__ __forceinline__ void hash_scatter_levels(const DevGrid &g, float *gt, float3 pos, int l0, const float (&dF)[2 * NL], int lane)
{
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        const int l = l0 + j;
        float ax = dF[2 * j], ay = dF[2 * j + 1];
        const float sc = g.scale[l];
        const float px = __fmaf_rn(sc, pos.x, 0.5f), py = __fmaf_rn(sc, pos.y, 0.5f), pz = __fmaf_rn(sc, pos.z, 0.5f);
        const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
        const uint32_t gx = (uint32_t)(int)fx, gy = (uint32_t)(int)fy, gz = (uint32_t)(int)fz;
        const float wx = __fsub_rn(px, fx), wy = __fsub_rn(py, fy), wz = __fsub_rn(pz, fz);
        float nwx = 0.f, nwy = 0.f, nwz = 0.f, nax = 0.f, nay = 0.f;
        bool take = false;
        if (l < SC_PAIR_LEVELS && sc < 60000.f) { /* cell coordinates below 2^16 */
            const uint32_t kxy = gx | (gy << 16);
            const uint32_t okxy = __shfl_xor_sync(FULLMASK, kxy, 1), okz = __shfl_xor_sync(FULLMASK, gz, 1);
            nwx = __shfl_xor_sync(FULLMASK, wx, 1);
            nwy = __shfl_xor_sync(FULLMASK, wy, 1);
            nwz = __shfl_xor_sync(FULLMASK, wz, 1);
            nax = __shfl_xor_sync(FULLMASK, ax, 1);
            nay = __shfl_xor_sync(FULLMASK, ay, 1);
            if (okxy == kxy && okz == gz) {
                if (lane & 1) ax = ay = 0.f;
                else take = nax != 0.f || nay != 0.f;
            }
        }
        if (ax == 0.f && ay == 0.f && !take) continue;
        const uint32_t size = g.size[l];
        float *tl = gt + 2 * (size_t)g.offset[l];
        const bool dense = (g.dense_mask >> l) & 1u;
        const bool even_off = (g.offset[l] & 1u) == 0u;
#pragma unroll
        for (int cp = 0; cp < 4; ++cp) {
            const uint32_t cy = gy + (cp & 1), cz = gz + (cp >> 1);
            uint32_t i0, i1;
            if (dense) {
                i0 = gx + cy * g.res[l] + cz * g.res2[l];
                if (i0 >= size) i0 -= size;
                i1 = i0 + 1u;
                if (i1 >= size) i1 -= size;
            } else {
                const uint32_t h = (cy * 2654435761u) ^ (cz * 805459861u);
                i0 = (gx ^ h) & (size - 1u);
                i1 = ((gx + 1u) ^ h) & (size - 1u);
            }
            const float wyz = ((cp & 1) ? wy : 1.0f - wy), wzz = ((cp & 2) ? wz : 1.0f - wz);
            const float w0 = ((1.0f - wx) * wyz) * wzz, w1 = (wx * wyz) * wzz;
            float v0x = w0 * ax, v0y = w0 * ay, v1x = w1 * ax, v1y = w1 * ay;
            if (take) {
                const float nyz = ((cp & 1) ? nwy : 1.0f - nwy), nzz = ((cp & 2) ? nwz : 1.0f - nwz);
                const float n0 = ((1.0f - nwx) * nyz) * nzz, n1 = (nwx * nyz) * nzz;
                v0x = fmaf(n0, nax, v0x); v0y = fmaf(n0, nay, v0y);
                v1x = fmaf(n1, nax, v1x); v1y = fmaf(n1, nay, v1y);
            }
            if ((i0 ^ i1) == 1u && even_off) {
                if (i0 & 1u) red_add4(tl + 2 * (size_t)i1, v1x, v1y, v0x, v0y);
                else red_add4(tl + 2 * (size_t)i0, v0x, v0y, v1x, v1y);
            } else {
                red_add2(tl + 2 * (size_t)i0, v0x, v0y);
                red_add2(tl + 2 * (size_t)i1, v1x, v1y);
            }
        }
    }
}

__device__ __forceinline__ void tmem_ld_n(uint32_t taddr, float (&v)[16]) { tmem_ld16(taddr, v); }
__device__ __forceinline__ void tmem_ld_n(uint32_t taddr, float (&v)[32]) { tmem_ld32(taddr, v); }

/* hash_encode restricted to levels l0 .. l0 + NL - 1, LG levels' gathers in
 * flight together; the same arithmetic, so the same features */
template <int NL, int LG>
__device__ __forceinline__ void encode_levels(const DevGrid &g, const __half2 *__restrict__ table, float3 pos, int l0, __half2 (&out)[NL])
{
#pragma unroll
    for (int j0 = 0; j0 < NL; j0 += LG) {
        __half2 v[LG][8];
        float wx[LG], wy[LG], wz[LG];
#pragma unroll
        for (int j = 0; j < LG; ++j) {
            const int l = l0 + j0 + j;
            const float sc = g.scale[l];
            const float px = __fmaf_rn(sc, pos.x, 0.5f), py = __fmaf_rn(sc, pos.y, 0.5f), pz = __fmaf_rn(sc, pos.z, 0.5f);
            const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
            const uint32_t gx = (uint32_t)(int)fx, gy = (uint32_t)(int)fy, gz = (uint32_t)(int)fz;
            wx[j] = __fsub_rn(px, fx); wy[j] = __fsub_rn(py, fy); wz[j] = __fsub_rn(pz, fz);
            const uint32_t size = g.size[l];
            const __half2 *tl = table + g.offset[l];
            if ((g.dense_mask >> l) & 1u) {
                const uint32_t rr = g.res[l], r2 = g.res2[l];
                const uint32_t b0 = gx + gy * rr + gz * r2;
                if (b0 + 1u + rr + r2 < size) { /* no corner reaches past the table */
#pragma unroll
                    for (int c = 0; c < 8; ++c) v[j][c] = __ldg(tl + (b0 + ((c & 1) ? 1u : 0u) + ((c & 2) ? rr : 0u) + ((c & 4) ? r2 : 0u)));
                } else {
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        uint32_t i = b0 + ((c & 1) ? 1u : 0u) + ((c & 2) ? rr : 0u) + ((c & 4) ? r2 : 0u);
                        if (i >= size) i -= size;
                        v[j][c] = __ldg(tl + i);
                    }
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
        for (int j = 0; j < LG; ++j) {
            float2 e[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) e[q] = f2_lerp(__half22float2(v[j][2 * q]), __half22float2(v[j][2 * q + 1]), wx[j]);
            const float2 g0 = f2_lerp(e[0], e[1], wy[j]), g1 = f2_lerp(e[2], e[3], wy[j]);
            out[j0 + j] = __float22half2_rn(f2_lerp(g0, g1, wz[j]));
        }
    }
}

template <int PREC, int HH>
__global__ void __launch_bounds__(BT_THREADS, 2) wf_net_bwd_tc_kernel(RenderParams p, BwdParams b, int it)
{
    extern __shared__ __align__(128) unsigned char bt_smem_raw[];
    BtSmem &S = *reinterpret_cast<BtSmem *>(bt_smem_raw);
    const int n_rows = p.counters[6];
    if (n_rows == 0) return;
    using T16 = E16<PREC>;
    constexpr bool BF = PREC == 1;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        mbar_init(&S.mbar, 1);
        mbar_init(&S.in_full[0], BT_HASH_THREADS);
        mbar_init(&S.in_full[1], BT_HASH_THREADS);
        mbar_init(&S.df_full, 1);
        mbar_init(&S.df_empty, BT_HASH_THREADS);
        mbar_arrive_expect_tx(&S.mbar, TB_BYTES);
        bulk_copy_g2s(S.W, b.wtc, TB_BYTES, &S.mbar);
    }
    if (warp == 0) tmem_alloc(&S.tmem_base, BT_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lrow = tmem + ((uint32_t)((warp & 3) * 32) << 16); /* this thread's TMEM lane */
    const int row = tid & 127;
    const int n_tiles = (n_rows + 127) / 128;
    const int n_mine = blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    bool ok = true;
    if (warp >= 4) {
        /* ================= hash warps ================= */
        /* thread 128 + h: row h & 127, levels l0 .. l0 + BT_NL - 1; the first set also writes SH and dout */
        const int l0 = ((tid - 128) >> 7) * BT_NL;
        const bool lead = l0 == 0;
        const RayState *states = p.states[it & 1];
        int r_prev = -1;
        float3 pos_prev = make_float3(0.f, 0.f, 0.f);
        for (int i = 0; i <= n_mine && ok; ++i) {
            int r = -1;
            float3 pos = make_float3(0.f, 0.f, 0.f);
            if (i < n_mine) {
                /* tile i into buffer i & 1 (its last reader, tile i - 2, finished before df_full of i - 2,
                 * which this loop waited for one iteration ago) */
                const int bb = i & 1;
                const int k = ((int)blockIdx.x + i * (int)gridDim.x) * 128 + row;
                r = k < n_rows ? p.grad_res_list[k] : -1;
                float4 dout = make_float4(0.f, 0.f, 0.f, 0.f);
                __half2 feat[BT_NL], sh[8];
#pragma unroll
                for (int q = 0; q < BT_NL; ++q) feat[q] = __floats2half2_rn(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
                if (r >= 0) {
                    const float4 pw = p.row_pay[r];
                    pos = make_float3(pw.x, pw.y, pw.z);
                    if (lead) {
                        dout = p.row_dout[r];
                        sh16(row_dir01(states, p.row_slot[r]), sh);
                    }
                    encode_levels<BT_NL, FVC_BT_HASH_GROUP>(p.grid, p.table, pos, l0, feat);
                }
                uint32_t f[BT_NL];
#pragma unroll
                for (int q = 0; q < BT_NL; ++q) {
                    const float2 v = __half22float2(feat[q]);
                    f[q] = PREC == 0 ? *reinterpret_cast<const uint32_t *>(&feat[q]) : T16::pack(v.x, v.y);
                }
#pragma unroll
                for (int c = 0; c < BT_NL / 4; ++c)
                    bt_st(S.F[bb], row, l0 / 4 + c, 32, make_uint4(f[4 * c], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3]));
                if (lead) {
                    uint32_t sv[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float2 v = __half22float2(sh[q]);
                        sv[q] = PREC == 0 ? *reinterpret_cast<const uint32_t *>(&sh[q]) : T16::pack(v.x, v.y);
                    }
                    bt_st(S.IN[bb], row, 1, 32, make_uint4(sv[0], sv[1], sv[2], sv[3]));
                    bt_st(S.IN[bb], row, 2, 32, make_uint4(sv[4], sv[5], sv[6], sv[7]));
                    const uint32_t one2 = T16::pack(1.0f, 1.0f);
                    bt_st(S.IN[bb], row, 3, 32, make_uint4(one2, one2, one2, one2));
                    S.dout[bb][row] = dout;
                }
                fence_proxy_async();
                mbar_arrive(&S.in_full[bb]);
            }
            if (i >= 1) {
                /* feature gradients of tile i - 1 -> table */
                bt_wait_on(&S.df_full, (uint32_t)((i - 1) & 1), ok);
                ok = __all_sync(FULLMASK, ok); /* the TMEM load and the scatter's shuffles take whole warps */
                if (!ok) break;
                float dF[2 * BT_NL];
                tmem_ld_n(lrow + BT_DF + 2 * l0, dF);
                tmem_wait_ld();
                tc_fence_before();
                mbar_arrive(&S.df_empty);
                if (r_prev < 0)
#pragma unroll
                    for (int q = 0; q < 2 * BT_NL; ++q) dF[q] = 0.f;
                hash_scatter_levels<BT_NL>(p.grid, b.g_table, pos_prev, l0, dF, tid & 31);
            }
            r_prev = r;
            pos_prev = pos;
        }
    } else {
        /* ================= MMA warps ================= */
        const int lo = p.latent_offset;
        uint32_t phase = 0;
        bt_wait_on(&S.mbar, phase, ok); /* the weights */
        phase ^= 1u;
        ok = bt_publish(ok); /* every decision to leave the loop is taken by all MMA threads together */
        uint8_t *last = HH == 2 ? S.A4 : S.A3;
        bool acc = false; /* dW accumulators hold this launch's sums */
#define BT_STAGE(...)                                   \
    if (tid == 0) {                                     \
        tc_fence_after();                               \
        __VA_ARGS__;                                    \
        tc_commit(&S.mbar);                             \
    }                                                   \
    bt_wait_on(&S.mbar, phase, ok);                     \
    phase ^= 1u;
        for (int i = 0; i < n_mine && ok; ++i) {
            const int bb = i & 1;
            uint8_t *F = S.F[bb], *IN = S.IN[bb];
            bt_wait_on(&S.in_full[bb], (uint32_t)((i >> 1) & 1), ok);
            const float4 dout = S.dout[bb][row];
            bt_st(S.G16, row, 0, 16, make_uint4(T16::pack(clamp_h(dout.x), clamp_h(dout.y)), T16::pack(clamp_h(dout.z), 0.f), 0u, 0u));
            bt_st(S.G16, row, 1, 16, make_uint4(0u, 0u, 0u, 0u));
            if (!(ok = bt_publish(ok))) break;
            /* ---- density layer 1: F W1^T -> H1 ---- */
            BT_STAGE(bt_mma_k(tmem + BT_D0, F, S.W + TB_W1, 32, 64, BF));
            bt_epi_act<PREC>(lrow + BT_D0, S.H1, row);
            if (!(ok = bt_publish(ok))) break;
            /* ---- density layer 2: H1 W2^T -> latents of the head input ---- */
            BT_STAGE(bt_mma_k(tmem + BT_D0, S.H1, S.W + TB_W2, 64, 16, BF));
            {
                float v[16];
                tmem_ld16(lrow + BT_D0, v);
                tmem_wait_ld();
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) /* latent_offset is 0 or 1 */
                    w[q] = T16::pack(clamp_h(lo ? v[2 * q + 1] : v[2 * q]), clamp_h(lo ? v[2 * q + 2] : v[2 * q + 1]));
                bt_st(IN, row, 0, 32, make_uint4(w[0], w[1], w[2], w[3]));
            }
            if (!(ok = bt_publish(ok))) break;
            /* ---- head layer 1 (bias from the 1-padding) -> A3 ---- */
            BT_STAGE(bt_mma_k(tmem + BT_D0, IN, S.W + TB_W3, 32, 64, BF));
            bt_epi_act<PREC>(lrow + BT_D0, S.A3, row);
            if (!(ok = bt_publish(ok))) break;
            if (HH == 2) {
                /* ---- head layer 2 -> A4 ---- */
                BT_STAGE(bt_mma_k(tmem + BT_D0, S.A3, S.W + TB_W4, 64, 64, BF));
                bt_epi_act<PREC>(lrow + BT_D0, S.A4, row);
                if (!(ok = bt_publish(ok))) break;
            }
            /* ---- output layer: G5 W5 -> gradient of the last hidden layer; dW5^T += last^T G5 ---- */
            BT_STAGE(bt_mma_kw(tmem + BT_D0, S.G16, S.W + TB_W5, 64, 16, 64, BF); bt_mma_mn(tmem + BT_DW5T, last, 64, S.G16, 16, BF, acc));
            bt_epi_grad<PREC>(lrow + BT_D0, last, row);
            if (!(ok = bt_publish(ok))) break;
            if (HH == 2) {
                /* ---- head layer 2: G4 W4 -> G3 (mask A3); dW4 += G4^T A3 ---- */
                BT_STAGE(bt_mma_kw(tmem + BT_D0, S.A4, S.W + TB_W4, 64, 64, 64, BF); bt_mma_mn(tmem + BT_DW4, S.A4, 64, S.A3, 64, BF, acc));
                bt_epi_grad<PREC>(lrow + BT_D0, S.A3, row);
                if (!(ok = bt_publish(ok))) break;
            }
            /* ---- head layer 1: G3 W3 -> latent gradients; dW3 += G3^T IN ---- */
            BT_STAGE(bt_mma_kw(tmem + BT_D0, S.A3, S.W + TB_W3, 32, 64, 16, BF); bt_mma_mn(tmem + BT_DW3, S.A3, 64, IN, 32, BF, acc));
            {
                float v[16];
                tmem_ld16(lrow + BT_D0, v);
                tmem_wait_ld();
                /* gradient of the density-network outputs: latents at lo.., the log-density gradient added to column 0 */
                float dl[8], gv[16];
#pragma unroll
                for (int j = 0; j < 8; ++j) dl[j] = T16::flt(T16::one(clamp_h(v[j])));
#pragma unroll
                for (int j = 0; j < 16; ++j) gv[j] = 0.f;
#pragma unroll
                for (int j = 0; j < 8; ++j) { /* latent_offset is 0 or 1 */
                    if (lo) gv[j + 1] = dl[j];
                    else gv[j] = dl[j];
                }
                gv[0] = clamp_h(gv[0] + dout.w);
                uint32_t w[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) w[q] = T16::pack(gv[2 * q], gv[2 * q + 1]);
                bt_st(S.G16, row, 0, 16, make_uint4(w[0], w[1], w[2], w[3]));
                bt_st(S.G16, row, 1, 16, make_uint4(w[4], w[5], w[6], w[7]));
            }
            if (!(ok = bt_publish(ok))) break;
            /* ---- density layer 2: G2 W2 -> G1 (mask H1); dW2^T += H1^T G2 ---- */
            BT_STAGE(bt_mma_kw(tmem + BT_D0, S.G16, S.W + TB_W2, 64, 16, 64, BF); bt_mma_mn(tmem + BT_DW2T, S.H1, 64, S.G16, 16, BF, acc));
            bt_epi_grad<PREC>(lrow + BT_D0, S.H1, row);
            if (!(ok = bt_publish(ok))) break;
            /* ---- density layer 1: G1 W1 -> feature gradients (for the hash warps); dW1 += G1^T F ---- */
            if (i >= 1) bt_wait_on(&S.df_empty, (uint32_t)((i - 1) & 1), ok); /* tile i - 1's gradients were read */
            if (!(ok = bt_publish(ok))) break;
            if (tid == 0) {
                tc_fence_after();
                bt_mma_kw(tmem + BT_DF, S.H1, S.W + TB_W1, 32, 64, 32, BF);
                bt_mma_mn(tmem + BT_DW1, S.H1, 64, F, 32, BF, acc);
                tc_commit(&S.df_full);
                tc_commit(&S.mbar);
            }
            bt_wait_on(&S.mbar, phase, ok);
            phase ^= 1u;
            acc = true;
            ok = bt_publish(ok);
        }
#undef BT_STAGE
        /* the CTA's weight gradients (TMEM lanes 0..63) into the global blobs */
        if (ok && acc && warp < 2) {
            float *gh = b.g_head, *gb = b.g_base;
            auto add_rows = [&](uint32_t col, float *dst, int width) { /* lane t = output o: dst[o * width + i] */
                for (int c0 = 0; c0 < width; c0 += 32) {
                    float v[32];
                    tmem_ld32(lrow + col + c0, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int q = 0; q < 32; ++q)
                        if (v[q] != 0.f) atomicAdd(dst + tid * width + c0 + q, v[q]);
                }
            };
            auto add_cols = [&](uint32_t col, float *dst) { /* lane t = input i: dst[o * 64 + i] */
                float v[16];
                tmem_ld16(lrow + col, v);
                tmem_wait_ld();
#pragma unroll
                for (int o = 0; o < 16; ++o)
                    if (v[o] != 0.f) atomicAdd(dst + o * 64 + tid, v[o]);
            };
            if (HH == 2) add_rows(BT_DW4, gh + GH_W4, 64);
            add_rows(BT_DW3, gh + GH_W3, 32);
            add_rows(BT_DW1, gb + GB_W1, 32);
            add_cols(BT_DW5T, gh + b.head_w5);
            add_cols(BT_DW2T, gb + GB_W2);
        }
    }
    if (!ok) atomicOr(p.guard, 16);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, BT_COLS);
    }
}

/* Cache rows of the cached differentiable render: the head input is the
 * trilinear blend of the 8 corner voxels' latents (divided by sum(w isset),
 * generateNetworkInput_cache_shfl_perf_kernel_cg), so the head's input
 * gradient goes to each corner with weight w_c / sum(w isset).  One warp per
 * 32 cache rows: lookup, head forward, head backward (weight gradients into
 * the per-CTA head blob), latent scatter with red.global.add.v2.f32.  The
 * voxel densities get no gradient. */
template <int PREC, int HH>
__global__ void __launch_bounds__(BW_WARPS * 32, 1) wf_cache_bwd_kernel(RenderParams p, BwdParams b, int it)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BwdSmem &S = *reinterpret_cast<BwdSmem *>(smem_raw);
    const int n_rows = p.counters[7];
    if (n_rows == 0) return;
    float *dWh = S.dW + GB_BASE;
    for (int i = threadIdx.x; i < DW_FLOATS - GB_BASE; i += blockDim.x) dWh[i] = 0.f;
    __syncthreads();
    using T16 = E16<PREC>;
    const int warp = threadIdx.x >> 5, lane = lane_id();
    BwdWarp &W = S.w[warp];
    const RayState *states = p.states[it & 1];
    uint16_t *inr = W.IN + lane * S32;
    uint16_t *gr = W.G + lane * S64;
    const int n_tiles = (n_rows + 31) / 32;
    const Voxel *voxels = reinterpret_cast<const Voxel *>(p.cache.voxels);
    for (int tile = blockIdx.x * BW_WARPS + warp; tile < n_tiles; tile += gridDim.x * BW_WARPS) {
        const int k = tile * 32 + lane;
        const int r = k < n_rows ? p.grad_cache_list[k] : -1;
        float4 dout = make_float4(0.f, 0.f, 0.f, 0.f);
        const Voxel *vp[8];
        float wc[8];
        float wsum = 0.f, ls[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        __half2 sh[8];
        if (r >= 0) {
            dout = p.row_dout[r];
            const float4 pw = p.row_pay[r];
            cache_corners(p.cache, make_float3(pw.x, pw.y, pw.z), vp, wc);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (!vp[c]) continue;
                float2 di;
                uint4 lt;
                ld_voxel(vp[c], di, lt);
                wsum = fmaf(wc[c], di.y, wsum);
                const uint32_t lw[4] = {lt.x, lt.y, lt.z, lt.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float2 fq = __half22float2(*reinterpret_cast<const __half2 *>(&lw[q]));
                    ls[2 * q] = fmaf(wc[c], fq.x, ls[2 * q]);
                    ls[2 * q + 1] = fmaf(wc[c], fq.y, ls[2 * q + 1]);
                }
            }
            sh16(row_dir01(states, p.row_slot[r]), sh);
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c) vp[c] = nullptr;
#pragma unroll
            for (int q = 0; q < 8; ++q) sh[q] = __floats2half2_rn(0.f, 0.f);
        }
        /* head input [latents (fp16 as the forward lookup rounds them) | SH | 1-padding] */
        const float inv = wsum != 0.f ? 1.0f / wsum : 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) inr[j] = T16::one(__half2float(__float2half_rn(ls[j] * inv)));
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float2 f = __half22float2(sh[q]);
            reinterpret_cast<uint32_t *>(inr + 8)[q] = PREC == 0 ? *reinterpret_cast<const uint32_t *>(&sh[q]) : T16::pack(f.x, f.y);
        }
#pragma unroll
        for (int q = 24; q < 32; ++q) inr[q] = T16::one(1.0f);
        __syncwarp();
        {
            float c[2][8][4];
            warp_mm<PREC, 32, 64>(W.IN, S32, b.w + BW_F3, lane, c);
            st_tile<PREC, 64>(W.A3, S64, c, lane, 1);
        }
        __syncwarp();
        const uint16_t *last = W.A3;
        if (HH == 2) {
            float c[2][8][4];
            warp_mm<PREC, 64, 64>(W.A3, S64, b.w + BW_F4, lane, c);
            st_tile<PREC, 64>(W.A4, S64, c, lane, 1);
            __syncwarp();
            last = W.A4;
        }
        gr[0] = T16::one(clamp_h(dout.x));
        gr[1] = T16::one(clamp_h(dout.y));
        gr[2] = T16::one(clamp_h(dout.z));
#pragma unroll
        for (int q = 3; q < 16; ++q) gr[q] = 0;
        __syncwarp();
        warp_dw<PREC, 16, 64>(W.G, S64, last, S64, dWh + b.head_w5, lane);
        {
            float c[2][8][4];
            warp_mm<PREC, 16, 64>(W.G, S64, b.w + BW_B5, lane, c);
            __syncwarp();
            st_tile<PREC, 64>(W.G, S64, c, lane, 2, last, S64);
        }
        __syncwarp();
        if (HH == 2) {
            warp_dw<PREC, 64, 64>(W.G, S64, W.A3, S64, dWh + GH_W4, lane);
            float c[2][8][4];
            warp_mm<PREC, 64, 64>(W.G, S64, b.w + BW_B4, lane, c);
            __syncwarp();
            st_tile<PREC, 64>(W.G, S64, c, lane, 2, W.A3, S64);
            __syncwarp();
        }
        warp_dw<PREC, 64, 32>(W.G, S64, W.IN, S32, dWh + GH_W3, lane);
        float dl[2][1][4];
        warp_mm<PREC, 64, 8>(W.G, S64, b.w + BW_B3, lane, dl);
        /* d latents of each row (fp32, in the A3 tile) -> the row's corners */
        float *dL = reinterpret_cast<float *>(W.A3);
        __syncwarp();
        {
            const int g = lane >> 2, q = lane & 3;
#pragma unroll
            for (int m = 0; m < 2; ++m)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    float *d = dL + (16 * m + g + 8 * h) * DF_STRIDE + 2 * q;
                    d[0] = dl[m][0][2 * h];
                    d[1] = dl[m][0][2 * h + 1];
                }
        }
        __syncwarp();
        if (r >= 0 && wsum != 0.f) {
            const float *dr = dL + lane * DF_STRIDE;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (!vp[c]) continue;
                const float f = wc[c] * inv;
                float *gl = b.g_lat + (size_t)(vp[c] - voxels) * 8;
#pragma unroll
                for (int j = 0; j < 8; j += 2) red_add2(gl + j, f * dr[j], f * dr[j + 1]);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    auto flush = [&](const float *src, float *dst, int n, int I) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int row = i / I, col = i - row * I;
            const float v = src[row * I + dw_col(row, col)];
            if (v != 0.f) atomicAdd(dst + i, v);
        }
    };
    flush(dWh + GH_W3, b.g_head + GH_W3, 64 * 32, 32);
    if (HH == 2) flush(dWh + GH_W4, b.g_head + GH_W4, 64 * 64, 64);
    flush(dWh + b.head_w5, b.g_head + b.head_w5, 16 * 64, 64);
}

/* per ray: squared error of the white-background pixel, dL/dC (loss-scaled,
 * without the 1/N of the mean) and X_total = g.C + g_T T */
__global__ void loss_kernel(RenderParams p, BwdParams b)
{
    double local = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n_list; i += gridDim.x * blockDim.x) {
        const float4 c = p.results[i];
        const float e0 = c.x + c.w - b.target[3 * i], e1 = c.y + c.w - b.target[3 * i + 1], e2 = c.z + c.w - b.target[3 * i + 2];
        local += (double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2;
        const float s = 2.0f * b.loss_scale;
        const float g0 = s * e0, g1 = s * e1, g2 = s * e2;
        const_cast<float4 *>(p.ray_grad)[i] = make_float4(g0, g1, g2, g0 * c.x + g1 * c.y + g2 * c.z + (g0 + g1 + g2) * c.w);
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(FULLMASK, local, o);
    __shared__ double part[8];
    if (lane_id() == 0) part[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        atomicAdd(b.loss, t);
    }
}

cudaError_t launch_loss(const RenderParams &p, const BwdParams &b, cudaStream_t s)
{
    const int blocks = std::min(1024, (p.n_list + 255) / 256);
    loss_kernel<<<std::max(1, blocks), 256, 0, s>>>(p, b);
    return cudaGetLastError();
}

cudaError_t launch_net_backward(const RenderParams &p, const BwdParams &b, int head_hidden, int it, int n_sms, cudaStream_t s)
{
    static PerDeviceOnce attrs;
    const int smem = (int)sizeof(BwdSmem);
    cudaError_t ea = attrs.run([smem] {
        cudaError_t e = cudaFuncSetAttribute(wf_net_bwd_kernel<0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_kernel<0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_kernel<1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_kernel<1, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        return e;
    });
    if (ea != cudaSuccess) return ea;
    const bool bf16 = p.precision == 1;
    if (p.use_tc) {
        static PerDeviceOnce tc_attrs;
        const int tsmem = (int)sizeof(BtSmem);
        ea = tc_attrs.run([tsmem] {
            cudaError_t e = cudaFuncSetAttribute(wf_net_bwd_tc_kernel<0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_tc_kernel<0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_tc_kernel<1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
            if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_tc_kernel<1, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem);
            return e;
        });
        if (ea != cudaSuccess) return ea;
        const int grid = 2 * n_sms;
        if (head_hidden == 2) {
            if (bf16) wf_net_bwd_tc_kernel<1, 2><<<grid, BT_THREADS, tsmem, s>>>(p, b, it);
            else wf_net_bwd_tc_kernel<0, 2><<<grid, BT_THREADS, tsmem, s>>>(p, b, it);
        } else {
            if (bf16) wf_net_bwd_tc_kernel<1, 1><<<grid, BT_THREADS, tsmem, s>>>(p, b, it);
            else wf_net_bwd_tc_kernel<0, 1><<<grid, BT_THREADS, tsmem, s>>>(p, b, it);
        }
        return cudaGetLastError();
    }
    if (head_hidden == 2) {
        if (bf16) wf_net_bwd_kernel<1, 2><<<n_sms, BW_WARPS * 32, smem, s>>>(p, b, it);
        else wf_net_bwd_kernel<0, 2><<<n_sms, BW_WARPS * 32, smem, s>>>(p, b, it);
    } else {
        if (bf16) wf_net_bwd_kernel<1, 1><<<n_sms, BW_WARPS * 32, smem, s>>>(p, b, it);
        else wf_net_bwd_kernel<0, 1><<<n_sms, BW_WARPS * 32, smem, s>>>(p, b, it);
    }
    return cudaGetLastError();
}

cudaError_t launch_cache_backward(const RenderParams &p, const BwdParams &b, int head_hidden, int it, int n_sms, cudaStream_t s)
{
    static PerDeviceOnce attrs;
    const int smem = (int)sizeof(BwdSmem);
    const cudaError_t ea = attrs.run([smem] {
        cudaError_t e = cudaFuncSetAttribute(wf_cache_bwd_kernel<0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_cache_bwd_kernel<0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        return e;
    });
    if (ea != cudaSuccess) return ea;
    if (head_hidden == 2) wf_cache_bwd_kernel<0, 2><<<n_sms, BW_WARPS * 32, smem, s>>>(p, b, it);
    else wf_cache_bwd_kernel<0, 1><<<n_sms, BW_WARPS * 32, smem, s>>>(p, b, it);
    return cudaGetLastError();
}

/* gradient read-out: out += scratch * inv_scale, scratch = 0 */
__global__ void grad_finalize_kernel(float *scratch, float *out, size_t n, float inv_scale)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float v = scratch[i];
        if (v != 0.f) {
            out[i] += v * inv_scale;
            scratch[i] = 0.f;
        }
    }
}

cudaError_t launch_grad_finalize(float *scratch, float *out, size_t n, float inv_scale, int n_sms, cudaStream_t s)
{
    const int blocks = (int)std::min<size_t>((size_t)n_sms * 8, (n + 255) / 256);
    grad_finalize_kernel<<<std::max(1, blocks), 256, 0, s>>>(scratch, out, n, inv_scale);
    return cudaGetLastError();
}

}  // namespace fvc
