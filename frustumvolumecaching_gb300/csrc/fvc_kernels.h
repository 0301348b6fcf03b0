/*
 * fvc_kernels.h - launch parameter blocks of the renderer's kernels.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "fvc_device.cuh"
#include "fvc_tc.cuh"

namespace fvc {

/* Runs a set-up step (kernel attributes: cudaFuncSetAttribute applies to the
 * current device only) once per device ordinal, with that device current. */
class PerDeviceOnce {
public:
    template <class F>
    cudaError_t run(F &&setup)
    {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lk(mu_);
        if (done_[dev]) return cudaSuccess;
        e = setup();
        if (e == cudaSuccess) done_[dev] = true;
        return e;
    }

private:
    static constexpr int kMaxDevices = 256;
    std::mutex mu_;
    bool done_[kMaxDevices] = {};
};

/* read-only view of a built frustum cache (Cache, include/cache.h:12-74):
 * packed brick index [bZ][bY][bX] (x fastest; pack3D(slot) or -1),
 * known_ranges_to [fH][fW], voxels [slots][512] of 32 bytes */
struct CacheView {
    const int32_t *packed_index;
    const float *known_ranges;
    const void *voxels;
    int fW, fH, fD, bX, bY, bZ, dX, dY, dZ;
    int n_valid_slots;          /* slots written by the last build; others read as zero */
    int interp;                 /* CacheSettings::interpol_function of the render (InterpolFunction) */
    int first_latent_is_density; /* interpol_variant DensityIntermediates: latent 0 holds the density */
    /* the rest of CacheSettings, read by the basic cache renderer */
    int variant, reweight, keep_first, inter_brick;
};

enum : int { INTERP_LINEAR = 0, INTERP_SMOOTHSTEP = 1, INTERP_SMOOTHERSTEP = 2, INTERP_NEAREST = 3 };
enum : int { VARIANT_DENSITY = 0, VARIANT_ALPHA = 1, VARIANT_INTERMEDIATES = 2, VARIANT_DENSITY_INTERMEDIATES = 3,
             VARIANT_ALPHA_INTERMEDIATES = 4 };

/* applyInterpolationFunction (include/raymarch_common.h:393-402) on one
 * trilinear fraction t in [0, 1): smoothstep t^2 (3 - 2t), smootherstep
 * t^3 (t (6t - 15) + 10) (include/util/helper_math_extension.h:146-181),
 * nearest = round half to even */
__device__ __forceinline__ float interp_weight(float t, int fn)
{
    if (fn == INTERP_SMOOTHSTEP) return (t * t) * (3.0f - 2.0f * t);
    if (fn == INTERP_SMOOTHERSTEP) return ((t * t) * t) * (t * (6.0f * t - 15.0f) + 10.0f);
    if (fn == INTERP_NEAREST) return rintf(t);
    return t;
}

/* weights of the tcgen05 network in canonical K-major tiles (bytes) */
constexpr int TC_B1 = 0;        /* 64 x 32 */
constexpr int TC_B2 = 4096;     /* 16 x 64 */
constexpr int TC_B3 = 6144;     /* 64 x 32 */
constexpr int TC_B4 = 10240;    /* 64 x 64 */
constexpr int TC_B5 = 18432;    /* 16 x 64 */
constexpr int TC_WBYTES = 20480;
/* a head with the positional frequency encoding (freq_encoding_degree 4,
 * include/nerf_network.h:55-81,241-246): its first layer reads K = 64 inputs
 * [density outputs 16 | SH 16 | 24 sines and cosines | 8 zero] */
constexpr int TCF_B3 = 6144;    /* 64 x 64 */
constexpr int TCF_B4 = 14336;   /* 64 x 64 */
constexpr int TCF_B5 = 22528;   /* 16 x 64 */
constexpr int TCF_WBYTES = 24576;
/* the view-dependent split network (NerfNetwork::init_viewdep,
 * include/nerf_network.h:120-158) as K-major tiles: density MLP, first head
 * ([density outputs | SH of the initial direction] 32 -> 64 -> 16 latent
 * rows), color head whose input is [latents 8 | SH 16 | SH difference 16 |
 * 1-padding 8] (K = 48) */
constexpr int VD_B1 = 0;        /* 64 x 32 */
constexpr int VD_B2 = 4096;     /* 16 x 64 */
constexpr int VD_F1 = 6144;     /* 64 x 32 */
constexpr int VD_F2 = 10240;    /* 16 x 64 */
constexpr int VD_B3 = 12288;    /* 64 x 48 */
constexpr int VD_B4 = 18432;    /* 64 x 64 */
constexpr int VD_B5 = 26624;    /* 16 x 64 */
constexpr int VD_WBYTES = 28672;
/* with the positional frequency encoding the color head reads [latents 8 | SH 16 | SH difference 16 |
 * frequency 24] (K = 64, no padding): its tiles shift */
constexpr int VDF_B4 = 20480;   /* 64 x 64 (VD_B3 holds 64 x 64) */
constexpr int VDF_B5 = 28672;   /* 16 x 64 */
constexpr int VDF_WBYTES = 30720;
/* the same in e4m3 (8-bit K-major tiles) for the FP8 network */
constexpr int TC8_B1 = 0, TC8_B2 = 2048, TC8_B3 = 3072, TC8_B4 = 5120, TC8_B5 = 9216, TC8_WBYTES = 10240;

/* voxel of the cache data array: density, isset, 2 pad words, 8 fp16 latents */
struct __align__(16) Voxel {
    float density, isset, pad0, pad1;
    uint4 lat;
};

/* One voxel's density, isset and latents by a single 32-byte load (one
 * sector, one load instruction instead of two; voxels sit at 32-byte
 * multiples of the 256-byte aligned data array).  Read-only path: the data
 * array does not change while a render reads it. */
__device__ __forceinline__ void ld_voxel(const Voxel *v, float2 &di, uint4 &lt)
{
    uint32_t a, b, c, d, e, f, g, h;
    asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(a), "=r"(b), "=r"(c), "=r"(d), "=r"(e), "=r"(f), "=r"(g), "=r"(h)
        : "l"(v));
    (void)c; (void)d; /* the two pad words */
    di = make_float2(__uint_as_float(a), __uint_as_float(b));
    lt = make_uint4(e, f, g, h);
}

enum : int { KIND_RESAMPLE = 0, KIND_CACHE = 1, KIND_DROP = 2, KIND_SKIP = 3 };
/* Why a cached render's sample is not a cache hit, kept in the upper bits of
 * its row kind (row_kind = kind | reason << 2) and counted by the compositing
 * kernel over the rows it composites or drops
 * (sample_cache_performance_kernel, src/cache_performance_renderer.cu:91-163;
 * sample_cache_kernel, src/cache_basic_renderer.cu:20-210). */
enum : int {
    REASON_NONE = 0,
    REASON_OUTSIDE_FOV = 1,   /* resampled: outside the cache camera's image */
    REASON_OUTSIDE_DEPTH = 2, /* resampled: inside the image, outside the froxel depth */
    REASON_BEFORE_NEAR = 3,   /* resampled: before the cache's near plane */
    REASON_BEYOND_KNOWN = 4,  /* resampled: beyond the pixel's known range (where its tile's build stopped) */
    REASON_BRICK_UNSET = 5,   /* dropped: the froxel's brick holds no slot */
    REASON_VOXEL_EMPTY = 6,   /* dropped: the voxel under the point holds no density (basic: not set) */
    REASON_ALPHA = 7,         /* dropped (basic renderer): interpolated alpha not above the threshold */
    N_REASONS = 8
};
__host__ __device__ constexpr int row_kind_of(int k) { return k & 3; }
__host__ __device__ constexpr int row_reason_of(int k) { return k >> 2; }

/* voxel (X, Y, Z) of the data array, or null outside it or in a slot the
 * last build did not write (the reference clears its arrays per build) */
__device__ __forceinline__ const Voxel *texel(const CacheView &c, int X, int Y, int Z)
{
    if (X < 0 || Y < 0 || Z < 0 || X >= c.dX * 8 || Y >= c.dY * 8 || Z >= c.dZ * 8) return nullptr;
    const int slot = (X >> 3) * (c.dY * c.dZ) + (Y >> 3) * c.dZ + (Z >> 3);
    if (slot >= c.n_valid_slots) return nullptr;
    return reinterpret_cast<const Voxel *>(c.voxels) + (size_t)slot * 512 + ((Z & 7) * 64 + (Y & 7) * 8 + (X & 7));
}

/* the 8 trilinear corners of froxel point f (unnormalised texel
 * coordinates, border -> none; include/util/cuda_readwrite_array.h:41-62):
 * voxel or null, and weight (generateNetworkInput_cache_shfl_perf_kernel_cg,
 * src/cache_performance_renderer.cu:678-787) */
__device__ __forceinline__ void cache_corners(const CacheView &C, float3 f, const Voxel *(&vp)[8], float (&w)[8])
{
    const float fx = F_SUB(f.x, 0.5f), fy = F_SUB(f.y, 0.5f), fz = F_SUB(f.z, 0.5f);
    const float x0 = floorf(fx), y0 = floorf(fy), z0 = floorf(fz);
    float lx = F_SUB(fx, x0), ly = F_SUB(fy, y0), lz = F_SUB(fz, z0);
    if (C.interp != INTERP_LINEAR) {
        lx = interp_weight(lx, C.interp);
        ly = interp_weight(ly, C.interp);
        lz = interp_weight(lz, C.interp);
    }
    /* all 8 corners inside the frustum and inside one brick (7 of 8 positions per axis): one brick-index
     * load instead of eight, the same voxels */
    if (x0 >= 0.f && y0 >= 0.f && z0 >= 0.f && x0 + 1.0f < (float)C.fW && y0 + 1.0f < (float)C.fH && z0 + 1.0f < (float)C.fD) {
        const int ix = (int)x0, iy = (int)y0, iz = (int)z0;
        if ((ix & 7) != 7 && (iy & 7) != 7 && (iz & 7) != 7) {
            const int packed = __ldg(C.packed_index + ((size_t)(iz >> 3) * C.bY + (iy >> 3)) * C.bX + (ix >> 3));
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
                w[c] = (ox ? lx : 1.0f - lx) * (oy ? ly : 1.0f - ly) * (oz ? lz : 1.0f - lz);
                vp[c] = packed >= 0 ? texel(C, ((packed >> 20) & 1023) * 8 + (ix & 7) + ox, ((packed >> 10) & 1023) * 8 + (iy & 7) + oy,
                                            (packed & 1023) * 8 + (iz & 7) + oz)
                                    : nullptr;
            }
            return;
        }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
        const float cx = x0 + (float)ox, cy = y0 + (float)oy, cz = z0 + (float)oz;
        vp[c] = nullptr;
        w[c] = (ox ? lx : 1.0f - lx) * (oy ? ly : 1.0f - ly) * (oz ? lz : 1.0f - lz);
        const bool inside = cx >= 0.f && cx < (float)C.fW && cy >= 0.f && cy < (float)C.fH && cz >= 0.f && cz < (float)C.fD;
        if (inside) {
            const int ix = (int)cx, iy = (int)cy, iz = (int)cz;
            const int bx = ix >> 3, by = iy >> 3, bz = iz >> 3;
            const int packed = __ldg(C.packed_index + ((size_t)bz * C.bY + by) * C.bX + bx);
            if (packed >= 0)
                vp[c] = texel(C, ((packed >> 20) & 1023) * 8 + (ix & 7), ((packed >> 10) & 1023) * 8 + (iy & 7),
                              (packed & 1023) * 8 + (iz & 7));
        }
    }
}

/* state of one alive ray between sub-iterations (96 bytes) */
struct __align__(16) RayState {
    float4 of;    /* origin, far */
    float4 dt;    /* direction, t1 (start of the next step) */
    float4 acc;   /* rgb, transmittance */
    float4 comp;  /* Kahan compensation of the rgb sums */
    int4 cnt;     /* pixel id, composited resample, composited cache, steps */
    int4 cnt2;    /* dropped, done flag, samples pushed, - */
};

struct RenderStatsDev {
    unsigned long long n_samples, n_resamples, n_cache_hits, n_dropped, n_steps;
    int n_rounds, pad;
    unsigned long long n_reason[N_REASONS]; /* composited or dropped rows per REASON_* (cached renderers) */
};

/* one view's frustum cache with the camera and step grid it was built for */
struct ViewCache {
    CacheView cache;
    DevCam ccam;
    DevSteps csteps;
};

struct RenderParams {
    DevScene scene;
    DevSteps steps;
    DevCam cam;
    DevGrid grid;
    const uint8_t *bits;        /* Morton occupancy bitfield */
    const __half2 *table;       /* hash tables, F = 2 */
    const uint2 *weights;       /* fragment-ordered MLP weights, W_TOTAL entries */
    const float *bias3;         /* head layer-1 bias from the 1-padding */
    const uint8_t *weights_tc;  /* the same weights as canonical K-major tiles (tcgen05) */
    int use_tc;                 /* 1: tcgen05 network kernels, 0: mma.sync */
    int precision;              /* plain-path MLP precision: 0 fp16, 1 bf16, 2 fp8-e4m3 (tcgen05 only) */
    const uint8_t *weights_tc_bf16; /* the tcgen05 tiles in bf16 */
    const uint8_t *weights_tc_fp8;  /* e4m3 tiles, each layer scaled by 448 / amax */
    const float *tc_fp8_iw;     /* per layer amax / 448 (undoes the weight scale) */
    int latent_offset;
    int *ray_counter;
    int *guard;
    RenderStatsDev *stats;
    float4 *results;            /* rgb, transmittance per pixel (may be null) */
    int4 *ray_counts;           /* per pixel: composited resample, composited cache, dropped, steps (may be null) */
    uchar4 *image;              /* progressive uchar4 image (may be null) */
    int sample_index;
    int max_rounds;
    int max_samples_per_ray;    /* 0 = unlimited */
    /* cached render */
    DevCam ccam;
    DevSteps csteps;
    CacheView cache;
    int render_mode;            /* 0 default, 1 only cache, 2 only resampled */
    /* wavefront buffers */
    RayState *states[2];        /* alive rays, ping-pong between sub-iterations */
    int2 *ray_rows;             /* per alive ray: first row, number of rows (in t order) */
    float *row_t0;              /* per row: t0 of the sample */
    int *row_slot;              /* per row: alive slot of its ray */
    uint8_t *row_kind;          /* per row: resample / cache / known empty / skipped */
    float4 *row_pay;            /* per row: contracted position or froxel point */
    uint2 *row_out;             /* per row: fp16 logits r, g, b and log-density */
    uint4 *row_lat;             /* per place in the cache list: the 8 looked-up head inputs from K = latent_offset (fp16) */
    int *res_list, *cache_list; /* row ids of the two network streams */
    int *counters;              /* [0], [1] alive rays (ping-pong), [2] rows, [3] resample, [4] cache */
    int row_capacity;           /* rows per sub-iteration */
    int steps_per_iter;         /* marching steps per ray and sub-iteration */
    int m_tile;                 /* rows per tcgen05 network tile on the plain path: 64, 128 (0 = 128) or 256 */
    int fused_classify;         /* cached renders: classification in the march, one network launch for all rows */
    int skip_empty;             /* the march skips occupancy lookups inside empty cells (exact: occupied_skip) */
    float *contrib_res, *contrib_cache; /* cached renders: per-pixel compositing weight of resample / cache samples (added) */
    int row_target;             /* compaction batch: rows per sub-iteration the march aims at, samples per ray
                                 * = clamp(row_target / alive rays, 1, S_ROWS) (0 = row_capacity) */
    int basic_cache;            /* 1: CacheBasicRenderer semantics for the cached rows (classify_basic) */
    int view_dependent;         /* split head (mlp_first_head): first head + SH-difference head input */
    int freq;                   /* the head's positional frequency encoding degree (0, or 4: the TCF_* tile layout) */
    const uint8_t *weights_vd;  /* VD_WBYTES of K-major tiles of the view-dependent network */
    /* batched views: rays of n_views cameras (device array), view v's pixel
     * (x, y) at ray id view_off[v] + y * W_v + x; view_off[n_views] = rays;
     * a ray's view is in its state's cnt2.w.  With view_caches, each view
     * renders against its own frustum cache instead of `cache`. */
    const ViewCache *view_caches;
    const DevCam *views;
    const int *view_off;
    int n_views;
    int max_iterations;         /* bound of the device-side sub-iteration loop */
    /* differentiable render */
    const int *pixel_list;      /* rays for these pixels (y * W + x) instead of the full image; ray id = list index */
    int n_list;
    const float4 *ray_grad;     /* per ray: dL/dC (loss-scaled) and X_total = g.C + g_T T */
    float4 *row_dout;           /* per row: dL/d rgb logits, dL/d log-density (loss-scaled) */
    int *grad_res_list;         /* rows with a gradient: resample rows (counters[6]) */
    int *grad_cache_list;       /*                       cache rows (counters[7]) */
};

/* Weights of the backward kernel: fragment packs (mma.sync m16n8k16 B
 * operands, frag_pack order) of each layer W (out x in) for the forward
 * recomputation (B[k][n] = W[n][k]) and for the input gradients
 * (B[k][n] = W[k][n]); head layer 1 in the model's input order
 * [latents | SH | 1-padding]. */
constexpr int BW_F1 = 0;                   /* W1 64 x 32 : 8 ntiles x 2 ksteps */
constexpr int BW_F2 = BW_F1 + 8 * 2 * 32;  /* W2 16 x 64 : 2 x 4 */
constexpr int BW_F3 = BW_F2 + 2 * 4 * 32;  /* W3 64 x 32 : 8 x 2 */
constexpr int BW_F4 = BW_F3 + 8 * 2 * 32;  /* W4 64 x 64 : 8 x 4 */
constexpr int BW_F5 = BW_F4 + 8 * 4 * 32;  /* W5 16 x 64 : 2 x 4 */
constexpr int BW_B5 = BW_F5 + 2 * 4 * 32;  /* W5^T pack: N = 64, K = 16 : 8 x 1 */
constexpr int BW_B4 = BW_B5 + 8 * 1 * 32;  /* W4: N = 64, K = 64 : 8 x 4 */
constexpr int BW_B3 = BW_B4 + 8 * 4 * 32;  /* W3: N = 32, K = 64 : 4 x 4 */
constexpr int BW_B2 = BW_B3 + 4 * 4 * 32;  /* W2: N = 64, K = 16 : 8 x 1 */
constexpr int BW_B1 = BW_B2 + 8 * 1 * 32;  /* W1: N = 32, K = 64 : 4 x 4 */
constexpr int BW_TOTAL = BW_B1 + 4 * 4 * 32;
/* gradient blob offsets (floats): the model file layouts */
constexpr int GB_W1 = 0, GB_W2 = 64 * 32, GB_BASE = GB_W2 + 16 * 64;
constexpr int GH_W3 = 0, GH_W4 = 64 * 32;

/* Weights of the tcgen05 backward kernel: each layer W (out x in) once, as a
 * canonical K-major tile [out][in] (bytes).  The forward MMAs read it as
 * B^T = W^T; the input-gradient MMAs read the same tile MN-major as B = W.
 * Head layer 1 in the model's input order [latents | SH | 1-padding]. */
constexpr int TB_W1 = 0;       /* 64 x 32 */
constexpr int TB_W2 = 4096;    /* 16 x 64 */
constexpr int TB_W3 = 6144;    /* 64 x 32 */
constexpr int TB_W4 = 10240;   /* 64 x 64 */
constexpr int TB_W5 = 18432;   /* 16 x 64 */
constexpr int TB_BYTES = 20480;

struct BwdParams {
    const uint8_t *wtc;         /* TB_BYTES of K-major weight tiles (tcgen05 backward) */
    const uint2 *w;             /* BW_TOTAL fragment entries */
    float *g_table;             /* [entries][2] fp32 */
    float *g_base;              /* GB_BASE floats */
    float *g_head;              /* head blob floats */
    int head_w5;                /* offset of W5 in the head blob */
    double *loss;               /* sum of squared pixel errors (device) */
    const float *target;        /* [n_list][3] */
    float loss_scale;           /* gradients carry this factor until read out */
    float *g_lat;               /* [slots][512][8] fp32 cache-latent gradients (cached path) */
};


struct InferenceParams {
    DevGrid grid;
    const __half2 *table;
    const uint2 *weights;
    const float *bias3;
    const float *pos;           /* [n][3] contracted */
    const float *dir;           /* [n][3] unit_to_01 or null (density only) */
    int n;
    float *out4;                /* [n][4] logits r,g,b, log-density (fp16 values) */
    float *base_out;            /* [n][16] density-network outputs or null */
    float *features;            /* [n][32] hash features or null */
};

struct CacheRay {
    float3 o, d;
    float far_, T;
    int alive;
};

struct CacheBuildParams {
    DevScene scene;
    DevSteps steps;
    DevCam cam;
    DevGrid grid;
    const uint8_t *bits;
    const __half2 *table;
    const uint2 *weights;
    int latent_offset;
    int variant;                /* CacheSettings::interpol_variant: what the voxels' density and latent 0 hold */
    int view_dependent;         /* latents from the first head on the build ray's direction */
    const uint2 *weights_fh;    /* the first head's W_L1 / W_L2 fragment packs */
    float4 *build_dirs;         /* per build row: unit_to_01 of its ray direction (view-dependent models) */
    const int *dir_slot;        /* or, when build_dirs is null: per row the alive slot of its ray ... */
    const RayState *dir_states; /* ... in these ray states (the per-ray fill) */
    int bX, bY, bZ, fW, fH, fD, dX, dY, dZ, capacity;
    CacheRay *rays;             /* [tiles][64] */
    int *block_step;            /* [tiles] */
    uint8_t *tile_alive;        /* [tiles] */
    int *alive_list, *alive_list_next;
    int *n_alive_tiles, *n_alive_next;
    int *tile_n_samples;        /* [alive idx] */
    uint8_t *tile_processed, *tile_need;
    int *tile_n_alive;
    void *voxels;               /* [slots][512] voxels */
    int32_t *packed_index;
    float *known_ranges;
    int *slot_counter;
    int *jobs;                  /* [2 * tiles]: (alive idx, slot) */
    int *n_jobs;
    int *guard;
    int max_search;
    /* rows of one build iteration (capacity: tiles x 512) */
    float4 *build_rows;         /* contracted sample position */
    __half *build_den;          /* log-density (fp16) */
    uint4 *build_lat;           /* 8 latents (fp16) */
    int *build_row_of;          /* [alive idx][step][ray]: row or -1 */
    int *build_row_counter;
};

/* One frame: ray generation, then sub-iterations of march / network /
 * compositing until no ray is alive.  Reads the alive count back every
 * `check_every` sub-iterations through h_pinned (page-locked, >= 1 int). */
/* Kernel accounting of one frame: every kernel the frame launched, and
 * (when `ev` holds 2 * cap events) a begin/end event pair recorded on the
 * launching stream around each resample network launch, the frame's
 * dominant kernel. */
struct LaunchLog {
    long long launches = 0;
    cudaEvent_t *ev = nullptr;
    int cap = 0;
    int n_timed = 0;
    int n_untimed = 0;
    int split = -1;  /* fvc_render_backward: timed launches before this index are the forward pass's */
};

/* The per-ray cache fill (CacheRenderer::initCache, src/cache_renderer.cu:
 * 571-928): the cache camera's own rays marched like a plain render, their
 * occupied samples through the density network, then per sub-iteration
 * pr_mark (bricks holding a visible sample), the deterministic per-column
 * slot reservation (pr_count / pr_scan / pr_reserve, then pr_zero clears the
 * new slots) and pr_write (voxels, termination, compaction, known ranges). */
struct PerRayFillParams {
    DevScene scene;
    DevSteps steps;
    int W, H;
    RayState *states[2];        /* the renderer's alive-ray states (ping-pong) */
    const int2 *ray_rows;       /* per alive ray: first row, row count */
    const float *row_t0;
    const __half *den;          /* per row: log-density (fp16) */
    const uint4 *lat;           /* per row: latents latent_offset + 0..7 (fp16) */
    int *counters;              /* the renderer's wavefront counters: [0], [1] alive rays (ping-pong) */
    uint8_t *flag;              /* [bZ][bY][bX]: brick marked in this sub-iteration */
    uint8_t *set;               /* [bZ][bY][bX]: brick holds a slot */
    int32_t *packed_index;      /* [bZ][bY][bX] */
    float *known_ranges;        /* [fH][fW] */
    void *voxels;               /* [slots][512] */
    int bX, bY, bZ, dX, dY, dZ, capacity, variant;
    int *slot_counter;          /* [0] slots reserved so far (overflowing ones included), [1] its value before this
                                   sub-iteration */
    int *col_count, *col_base;  /* per brick column (bY x bX) */
};

__global__ void pr_known_init_kernel(PerRayFillParams p);
__global__ void pr_mark_kernel(PerRayFillParams p, int it);
__global__ void pr_count_kernel(PerRayFillParams p);
__global__ void pr_scan_kernel(PerRayFillParams p);
__global__ void pr_reserve_kernel(PerRayFillParams p);
__global__ void pr_zero_kernel(PerRayFillParams p);
__global__ void pr_write_kernel(PerRayFillParams p, int it);
cudaError_t launch_fill_march(const RenderParams &p, int it, int n_sms, cudaStream_t s);
cudaError_t launch_div_selftest(const float *x, const float *d, int n, float *q, float *ieee);
cudaError_t launch_wait_selftest(long long limit_cycles, long long *d_out, cudaStream_t s);
cudaError_t launch_fill_raygen(const RenderParams &p, cudaStream_t s);

cudaError_t render_frame(const RenderParams &p, bool cached, int head_hidden, int n_sms, cudaStream_t s, int *h_pinned,
                         int check_every, int *n_iterations, LaunchLog *log = nullptr);

/* The plain render of p.views as one CUDA graph: counter resets, raygen, and
 * a conditional WHILE node whose body runs two sub-iterations and then lets
 * the device decide whether rays are still alive (at most p.max_iterations
 * sub-iterations; the iteration count is left in p.counters[5]).  The graph
 * holds p by value: it is valid while the buffers p points to are. */
cudaError_t build_batch_graph(const RenderParams &p, bool cached, int head_hidden, int n_sms, cudaStream_t s, int n_rays,
                              cudaGraphExec_t *exec, int *n_kernels);

/* differentiable render (fvc_backward.cu): pass 1 is render_frame over p.pixel_list */
cudaError_t backward_frame(const RenderParams &p, const BwdParams &b, bool cached, int head_hidden, int n_sms, cudaStream_t s,
                           int *h_pinned, int check_every, LaunchLog *log = nullptr);
cudaError_t launch_loss(const RenderParams &p, const BwdParams &b, cudaStream_t s);
cudaError_t launch_net_backward(const RenderParams &p, const BwdParams &b, int head_hidden, int it, int n_sms, cudaStream_t s);
cudaError_t launch_cache_backward(const RenderParams &p, const BwdParams &b, int head_hidden, int it, int n_sms, cudaStream_t s);
cudaError_t launch_grad_finalize(float *scratch, float *out, size_t n, float inv_scale, int n_sms, cudaStream_t s);
cudaError_t launch_inference(const InferenceParams &p, int head_hidden, int n_sms, cudaStream_t s);

__global__ void cache_init_kernel(CacheBuildParams p);
cudaError_t launch_cache_search(const CacheBuildParams &p, int grid, cudaStream_t s);
cudaError_t launch_cache_density(const CacheBuildParams &p, int grid, cudaStream_t s);
/* the density network of a build iteration on tcgen05 (models without a first head) */
cudaError_t launch_cache_density_tc(const CacheBuildParams &p, const uint8_t *weights_tc, int n_sms, cudaStream_t s);
__global__ void cache_composite_kernel(CacheBuildParams p);
__global__ void cache_assign_kernel(CacheBuildParams p);
__global__ void cache_fill_kernel(CacheBuildParams p);
__global__ void cache_known_ranges_kernel(CacheBuildParams p);
__global__ void cache_compact_kernel(CacheBuildParams p, int n_tiles);

}  // namespace fvc
