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
 * Network backward, one warp per 32 rows (mma.sync m16n8k16, fp16 or bf16
 * operands like the forward MLP, fp32 accumulation): the forward activations of the rows (hash features,
 * density hidden layer, head input [latents | SH | 1-padding], head hidden
 * layers) are recomputed into shared memory; the gradient tile then walks
 * back through the layers.  Input gradients are tile x weight-pack products;
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
                const float2 di = __ldg(reinterpret_cast<const float2 *>(vp[c]));
                const uint4 lt = __ldg(&vp[c]->lat);
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
    static bool attrs = false;
    const int smem = (int)sizeof(BwdSmem);
    if (!attrs) {
        cudaError_t e = cudaFuncSetAttribute(wf_net_bwd_kernel<0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_kernel<0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_kernel<1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_net_bwd_kernel<1, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attrs = true;
    }
    const bool bf16 = p.precision == 1;
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
    static bool attrs = false;
    const int smem = (int)sizeof(BwdSmem);
    if (!attrs) {
        cudaError_t e = cudaFuncSetAttribute(wf_cache_bwd_kernel<0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wf_cache_bwd_kernel<0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attrs = true;
    }
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
