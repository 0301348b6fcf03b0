/*
 * fvc.h - C ABI of the GB300 frustum-volume-caching NeRF renderer.
 *
 * Plain C (no CUDA, no torch types): every entry point takes plain pointers,
 * sizes and POD structs, returns an int status (FVC_OK == 0) and records a
 * thread-local message readable through fvc_last_error().
 *
 * The POD structs below have the byte layout of the reference's own structs
 * (include/common.h:22-62 CameraMatrix, :74-91 SceneInfo, :93-164 StepsizeInfo,
 * :166-195 CameraInfo, :210-218 RaymarchInfo; include/renderer_common.h:74-78
 * BaseRayResult), so a caller holding the reference types can pass them by
 * pointer unchanged.  fvc_abi.cpp static_asserts every size and offset.
 *
 * Each function names the reference interface it replaces.  Renderers render
 * synchronously on their stream (the reference's render() is synchronous:
 * src/performance_renderer.cu:283 CUDA_SYNC_CHECK_THROW); device-pointer
 * variants (suffix _device) enqueue on the renderer's stream and return
 * without synchronising, so a caller can time them with its own events.
 */
#ifndef FVC_H
#define FVC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FVC_ALIGN(n) __attribute__((aligned(n)))
#else
#define FVC_ALIGN(n)
#endif

/* ---- status codes (reference: exceptions / bool returns, see each fn) ---- */
#define FVC_OK 0
#define FVC_ERR_CUDA 1          /* a CUDA runtime call failed                  */
#define FVC_ERR_CONFIG 2        /* unsupported / malformed model or settings   */
#define FVC_ERR_OOM 3           /* device allocation failed                    */
#define FVC_ERR_CACHE_UNINIT 4  /* "Cache is not initialized!"                 */
#define FVC_ERR_TIMEOUT 5       /* a bounded device wait ran out               */
#define FVC_ERR_ARG 6           /* null handle / bad size / bad pointer        */
#define FVC_ERR_IO 7            /* model file missing or truncated             */
#define FVC_ERR_GUARD 8         /* a device-side guard fired (see message)     */

/* ---- vector PODs with CUDA's alignment (float2/int2: 8, float4: 16) ---- */
typedef struct FVC_ALIGN(8) { float x, y; } fvc_float2;
typedef struct { float x, y, z; } fvc_float3;
typedef struct FVC_ALIGN(16) { float x, y, z, w; } fvc_float4;
typedef struct FVC_ALIGN(8) { int x, y; } fvc_int2;
typedef struct { int x, y, z; } fvc_int3;

/* CameraMatrix, include/common.h:22-62: 3x4 row-major [R|t]. */
typedef struct { fvc_float4 m0, m1, m2; } fvc_camera_matrix;

/* ContractionType, include/common.h:66-72. */
enum { FVC_CONTRACTION_NONE = 0, FVC_CONTRACTION_AABB = 1,
       FVC_CONTRACTION_WARP_AABB_L2 = 2, FVC_CONTRACTION_WARP_AABB_LINF = 3 };

/* SceneInfo, include/common.h:74-91 (bool = 1 byte). */
typedef struct {
    int grid_resolution;
    int grid_nlvl;
    int vals_per_lvl;
    uint8_t normalized;
    fvc_float3 aabb_from;
    fvc_float3 aabb_to;
    fvc_float3 contraction_aabb_from;
    fvc_float3 contraction_aabb_to;
    int contraction_type;
    uint8_t is_open_gl;
    float alpha_thre;
} fvc_scene_info;

/* StepsizeInfo, include/common.h:93-164. */
typedef struct {
    float cone_angle, log1p_c, stepsize, near_, near_i, far_;
    float dt_min, dt_max, t_min, t_max, i_min, i_max;
} fvc_stepsize_info;

/* CameraInfo, include/common.h:166-195. */
typedef struct {
    fvc_int2 resolution;
    uint8_t is_open_gl;
    fvc_float2 focal;
    fvc_float2 principal;
    fvc_camera_matrix cam2world;
    fvc_camera_matrix world2cam;
    float aperature;
    float focus_z;
} fvc_camera_info;

/* RaymarchInfo, include/common.h:210-218. */
typedef struct {
    fvc_camera_info cam_info;
    fvc_camera_info next_cam_info;
    fvc_stepsize_info stepsize_info;
    int sample_index;
    uint8_t motion_blur;
    uint8_t deterministic;
} fvc_raymarch_info;

/* BaseRayResult, include/renderer_common.h:74-78 (rgb + transmittance). */
typedef struct FVC_ALIGN(16) { float r, g, b, transmittance; } fvc_ray_result;

/* CacheSettings, include/cache_renderer.h:24-32 (enum fields as int). */
typedef struct {
    int interpol_variant;      /* DensityInterpolVariant: 0 Density, 1 Alpha, 3 DensityIntermediates,
                                  4 AlphaIntermediates (2 Intermediates -> FVC_ERR_CONFIG) */
    int interpol_function;     /* InterpolFunction (include/common.h:221-227): 0 Linear, 1 Smoothstep,
                                  2 Smootherstep, 3 Nearest */
    uint8_t use_hw_interpol;
    uint8_t reweight_intermediates;
    uint8_t disable_reweighting_first_intermediate;
    uint8_t use_inter_brick_interpolation;
} fvc_cache_settings;

/* Renderer kinds: include/basic_renderer.h, performance_renderer.h,
 * cache_performance_renderer.h, cache_basic_renderer.h. BASIC shares the
 * PERFORMANCE kernels; CACHE_BASIC the cached ones, with the basic
 * renderer's per-sample cache semantics (isset decides, every CacheSettings
 * field applies, cache samples composite with their looked-up density). */
enum { FVC_RENDERER_BASIC = 0, FVC_RENDERER_PERFORMANCE = 1, FVC_RENDERER_CACHE_PERFORMANCE = 2, FVC_RENDERER_CACHE_BASIC = 3 };

/* Cache render modes: CachePerformanceRenderer::RenderMode
 * (include/cache_performance_renderer.h). */
enum { FVC_RENDER_MODE_DEFAULT = 0, FVC_RENDER_MODE_ONLY_CACHE = 1, FVC_RENDER_MODE_ONLY_RESAMPLED = 2 };

typedef struct fvc_model fvc_model;
typedef struct fvc_renderer fvc_renderer;
typedef struct fvc_cache fvc_cache;

/* Per-frame statistics: PerformanceRenderer::RenderStats and
 * CachePerformanceRenderer::RenderStats / CacheRenderer::InitStats
 * (include/performance_renderer.h:60-64, include/cache_renderer.h:104-109). */
typedef struct {
    double samples_ppx;              /* evaluated samples per pixel          */
    long long n_samples;             /* samples evaluated (resample + cache) */
    long long n_resamples;           /* samples through the full network     */
    long long n_cache_hits;          /* samples served from the cache        */
    long long n_dropped;             /* known-empty cache voxels skipped     */
    long long n_steps;               /* marching steps taken                 */
    int n_rounds;                    /* sub-iterations of the last render */
    int guard_flags;                 /* device guard bits (0 = none fired)   */
    long long n_launches;            /* kernels launched by the last render  */
    int n_timed_launches;            /* resample network launches timed      */
    float timed_kernel_ms;           /* their summed event time (0 = off)    */
    /* Cached renderers: why samples were not served by the cache, over the
     * samples composited or dropped (no counterpart in the reference, whose
     * _render_stats keep only the totals).  A sample outside several tests
     * counts under the first in the order image, near plane, known range,
     * froxel depth.  Resampled: */
    long long n_miss_outside_fov;    /* outside the cache camera's image         */
    long long n_miss_outside_depth;  /* in the image, outside the froxel depth   */
    long long n_miss_before_near;    /* before the cache's near plane            */
    long long n_miss_beyond_known;   /* beyond the pixel's known range: where its
                                      * tile's build stopped (opacity, the frustum
                                      * depth, or no slot left)                  */
    /* dropped: */
    long long n_drop_brick_unset;    /* the froxel's brick holds no slot         */
    long long n_drop_voxel_empty;    /* the voxel under the point holds no density
                                      * (basic renderer: is not set)             */
    long long n_drop_alpha;          /* basic renderer: interpolated alpha not
                                      * above the threshold                      */
    /* fvc_render_backward with kernel timing on: the network adjoint's
     * launches and their summed event time (the forward pass's network
     * launches stay in n_timed_launches / timed_kernel_ms) */
    int n_timed_adjoint_launches;
    float timed_adjoint_ms;
} fvc_render_stats_t;

typedef struct {
    int n_bricks_set;       /* bricks holding data                       */
    int n_bricks_reserved;  /* brick capacity of the data array          */
    int n_bricks_demanded;  /* allocations requested incl. overflowed    */
    int overflow;           /* 1 if at least one allocation overflowed   */
    int n_iterations;       /* depth-brick iterations of the build       */
    int n_launches;         /* kernels launched by the build             */
    long long n_samples;    /* samples evaluated by the density network  */
} fvc_cache_stats_t;

/* ------------------------------------------------------------------------ */
/* errors                                                                    */
/* ------------------------------------------------------------------------ */

/* Thread-local message of the last failing call (reference: the what() of the
 * std::runtime_error thrown by MY_CUDA_CHECK_THROW, include/util/cuda_helper.h:20-45). */
const char *fvc_last_error(void);
/* Library version string. */
const char *fvc_version(void);

/* ------------------------------------------------------------------------ */
/* model (reference: bool load_data(fs::path, LoaderData&), include/loader.h:49,   */
/* src/loader.cu:146-300): a path ending in ".ingp" is an instant-ngp snapshot */
/* (load_ingp_snapshot), any other path a nerfacc export directory            */
/* (load_nerfacc_export: config.json + *.dat).  An export whose config has    */
/* mlp_first_head loads as the view-dependent split network                  */
/* (NerfNetwork::init_viewdep, src/loader.cu:251-262); the renderers and     */
/* cache builds take it on the tcgen05 FP16 network path, the other paths    */
/* return FVC_ERR_CONFIG.                                                    */
/* ------------------------------------------------------------------------ */
int fvc_model_load(const char *data_dir, fvc_model **out);
/* Host only (no device work): the .ingp snapshot rewritten as the equivalent
 * nerfacc export directory - the scene, step and network configuration that
 * load_ingp_snapshot derives (src/loader.cu:176-213), the parameter blob split
 * into hash grid / density MLP / color MLP, and the occupancy grid thresholded
 * from the density grid (:73-114).  Loading the directory renders the same as
 * loading the snapshot. */
int fvc_ingp_export(const char *snapshot, const char *export_dir);
void fvc_model_destroy(fvc_model *m);
/* Scene and step parameters of the loaded model (LoaderData::scene_info,
 * ::stepsize_info after StepsizeInfo::setAdditionalInfo, include/common.h:109-131). */
int fvc_model_info(const fvc_model *m, fvc_scene_info *scene, fvc_stepsize_info *steps);
/* Failure-path checks (no counterpart in the reference).
 * fvc_debug_fail_allocation(n): the library's next n device allocations
 * succeed and the one after fails with FVC_ERR_OOM, as a full device would
 * make it fail (-1: off).  The call that hit it returns the error and leaves
 * the handle usable; a later call allocates again.
 * fvc_selftest_wait_timeout: runs the kernels' bounded device wait on an
 * mbarrier that nothing completes, with a limit of limit_ms; returns
 * FVC_ERR_TIMEOUT once the wait gave up (the normal outcome) with the time
 * waited, and leaves the CUDA context usable.  The network kernels use the
 * same wait (about 1 s) and report a run-out through the render guard. */
int fvc_debug_fail_allocation(long long n);
int fvc_selftest_wait_timeout(double limit_ms, double *waited_ms);
/* The kernels' exact division by a known denominator (Markstein's
 * correction of x * RN(1/d)) and the hardware IEEE division on n host pairs:
 * q[i] and q_ieee[i], for the tests that check they agree bit for bit. */
int fvc_selftest_division(const float *x, const float *d, int n, float *q, float *q_ieee);
/* StepsizeInfo::setAdditionalInfo (include/common.h:109-131): fills the
 * derived fields (dt_min/max, t_min/max, i_min/max, log1p_c, near_i) from
 * cone_angle, stepsize, near and far for the scene's grid.  Used by
 * StepsizeInfo::changeSamplingRate (include/common.h:130-135), e.g. a cache
 * built at twice the render's sampling rate. */
int fvc_stepsize_setup(const fvc_scene_info *scene, fvc_stepsize_info *steps);

/* Network and occupancy-grid properties a caller of the reference reads from
 * NerfNetwork / LoaderData: m_first_latent_is_density (include/nerf_network.h:342),
 * the head depth, and the device Morton bitfield (LoaderData::
 * occupancy_grid_morton_bitfield, include/loader.h:46; R^3 * nlvl / 8 bytes). */
typedef struct {
    int first_latent_is_density;
    int head_hidden_layers;
    int n_levels;
    int n_latents;
    const uint8_t *occupancy_bitfield;
    size_t occupancy_bytes;
} fvc_model_props;
int fvc_model_properties(const fvc_model *m, fvc_model_props *out);
/* Evaluate log-density (fp16-rounded density-network row 0) at n contracted
 * positions pos[3*n] in [0,1]^3 (NerfNetwork::inferenceLatents row 0,
 * include/nerf_network.h:173-202). Host buffers. */
int fvc_model_density(fvc_model *m, const float *pos, int n, float *log_density_out);
/* Full network at n samples: pos[3n] contracted, dir01[3n] = unit_to_01(dir);
 * out[4n] = (rgb logits 0..2, log-density) as fp16-rounded floats
 * (NerfNetwork::inference, include/nerf_network.h:160-171). Host buffers. */
int fvc_model_inference(fvc_model *m, const float *pos, const float *dir01, int n, float *out);

/* Diagnostics: hash-grid features features32[32n] and density-network
 * outputs base_out16[16n] (fp16 values) at n contracted positions; either
 * output may be NULL.  No reference counterpart (tcnn-internal values). */
int fvc_model_debug_encode(fvc_model *m, const float *pos, int n, float *features32, float *base_out16);

/* ------------------------------------------------------------------------ */
/* renderers (reference: Renderer / PerformanceRenderer / CachePerformanceRenderer */
/* constructors and virtual render / resizeRenderbuffers,                      */
/* include/renderer.h:108-112, include/performance_renderer.h:22-26)          */
/* ------------------------------------------------------------------------ */
int fvc_renderer_create(fvc_model *m, int kind, fvc_renderer **out);
void fvc_renderer_destroy(fvc_renderer *r);
/* resizeRenderbuffers(int2), src/performance_renderer.cu:186-212. */
int fvc_renderer_resize(fvc_renderer *r, int width, int height);
/* Use the caller's CUDA stream (cudaStream_t as void*; NULL = internal stream). */
int fvc_renderer_set_stream(fvc_renderer *r, void *cuda_stream);

/* Output buffers of a render; any member may be NULL.
 *   image_rgba8 [W*H*4]  uchar4 image after writeImageBuffer_performance_kernel
 *                        (white background, progressive average over
 *                        sample_index, src/performance_renderer.cu:127-149)
 *   results     [W*H]    rgb + transmittance before background / quantisation
 *                        (the final BaseRayResult of each ray)
 *   ray_counts  [W*H*4]  per ray: composited resample samples, composited
 *                        cache samples, known-empty cache voxels skipped,
 *                        marching steps */
typedef struct {
    uint8_t *image_rgba8;
    fvc_ray_result *results;
    int32_t *ray_counts;
    /* cache renderers, fvc_render_device only: per pixel, the compositing
     * weight (alpha T) the frame's resampled samples and its cache samples
     * contributed, ADDED to the device float buffers' contents (W x H each;
     * the caller clears them) - accumulate_cache_perf_kernel<DEBUG>'s
     * contribution surfaces (src/cache_performance_renderer.cu:789-908),
     * eval's -wc images.  NULL: not written. */
    float *contrib_resample;
    float *contrib_cache;
} fvc_render_outputs;

/* render(RaymarchInfo, RenderBuffer&, DebugData*) of the renderer's kind:
 * PerformanceRenderer::render (src/performance_renderer.cu:214-286) or
 * CachePerformanceRenderer::render (src/cache_performance_renderer.cu:1059-1263).
 * Device pointers.  The sub-iterations are enqueued on the renderer stream;
 * the host reads the alive-ray count back every 4 sub-iterations, so the
 * call returns once the last sub-iteration is enqueued (the final writes may
 * still be in flight on the stream). */
int fvc_render_device(fvc_renderer *r, const fvc_raymarch_info *info, const fvc_render_outputs *out);
/* Same with host pointers: H2D of the previous image (progressive average),
 * render, D2H of the outputs, synchronise. */
int fvc_render(fvc_renderer *r, const fvc_raymarch_info *info, const fvc_render_outputs *out);

/* Block until everything enqueued on the renderer's stream finished (the
 * reference's render() ends with CUDA_SYNC_CHECK_THROW,
 * src/performance_renderer.cu:283); reports a device guard as FVC_ERR_GUARD. */
int fvc_renderer_synchronize(fvc_renderer *r);
/* Guard on the samples of one ray (0 = off, the reference default); a ray
 * exceeding it sets a guard bit reported by fvc_render_stats. */
int fvc_renderer_set_max_samples_per_ray(fvc_renderer *r, int max_samples);
/* Network kernels of the renderer: 1 = 5th-generation tensor cores
 * (tcgen05.mma, TMEM accumulators; the default), 0 = warp-level mma.sync.
 * Both compute the same layers in fp16 with fp32 accumulation.  No reference
 * counterpart (the reference runs tiny-cuda-nn's FullyFusedMLP). */
int fvc_renderer_set_network_path(fvc_renderer *r, int use_tcgen05);
/* Density network of the cache builds (the blockwise build and the per-ray
 * fill; inferenceLatents, src/cache_renderer.cu:1020-1030, :893-900):
 * 0 = warp-level mma.sync (the default: these two layers on 32-row warp
 * tiles measured faster than 128-row tcgen05 tiles, whose per-layer
 * CTA-wide round trips the short network does not amortise), 1 = tcgen05.
 * View-dependent models build on mma.sync.  Slots, known ranges and isset
 * flags do not depend on it; voxel values agree to fp16 rounding.  No
 * reference counterpart. */
int fvc_renderer_set_build_network_path(fvc_renderer *r, int use_tcgen05);

/* Rows per tcgen05 network tile of the plain path (64, 128 or 256; FP16, not
 * view-dependent; default 128) and the compaction batch, the rows per
 * sub-iteration the march aims at (0: the renderer's row capacity, the
 * default; else in [2^10, 2^26], capped at the capacity).  Results do not
 * depend on either: every row's arithmetic is the same. */
int fvc_renderer_set_tiling(fvc_renderer *r, int m_tile, int batch_rows);

/* Cache renderers (CACHE_PERFORMANCE, tcgen05 path, density head): 1 (the
 * default) classifies each sample inside the march and runs one network
 * launch over all rows of a sub-iteration, a resample row gathering its hash
 * features and a cache row its trilinear lookup; 0 keeps the separate
 * classification pass with a resample list and a cache list.  The results
 * are the same bit for bit; the switch is for measurement. */
int fvc_renderer_set_fused_classify(fvc_renderer *r, int on);

/* Empty-space skipping in the renderers' march: 1 looks the occupancy grid
 * up once per empty cell at least four steps long and steps through the rest
 * of the cell without lookups (a DDA bound on the cell's extent along the
 * ray, as grid_occupied_at's t_dist_to_next_voxel,
 * include/raymarch_common.h:712-744, kept a margin inside the cell so every
 * step and occupancy decision is the plain march's); 0 (the default) looks up
 * every step.  Results are identical; on GB300 the skip measured slower
 * (the 32 rays of a warp seldom skip the same steps, so the lookups still
 * issue while the bound costs extra). */
int fvc_renderer_set_empty_space_skipping(fvc_renderer *r, int on);

/* MLP precision of the plain renderers on the tcgen05 path (no counterpart
 * in the reference, whose MLPs are fp16): FP16 (default), BF16, or
 * FP8-E4M3 with per-layer weight scaling and per-row activation scaling;
 * fp32 accumulation and fp32 Kahan-compensated compositing in every case. */
enum { FVC_PRECISION_FP16 = 0, FVC_PRECISION_BF16 = 1, FVC_PRECISION_FP8_E4M3 = 2 };
int fvc_renderer_set_precision(fvc_renderer *r, int precision);
/* Statistics of the last render (needs the stream synchronised). */
int fvc_render_stats(fvc_renderer *r, fvc_render_stats_t *out);

/* Record a CUDA event pair on the renderer's stream around every resample
 * network launch of the following renders (up to 4096 per render), summed
 * into fvc_render_stats.timed_kernel_ms.  No counterpart in the reference
 * (its timers wrap whole phases, include/renderer.h:79-105); used by the
 * benchmark to time the dominant kernel on its own stream. */
int fvc_renderer_set_kernel_timing(fvc_renderer *r, int enable);

/* Render without allocating (no counterpart in the reference).  For callers
 * that cannot call cudaMalloc while rendering (a host with its own fixed GPU
 * memory budget or allocator, per-frame callbacks with hard deadlines): the
 * plain render of PerformanceRenderer with all scratch in one file-scope
 * device array of FVC_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until exit.  Images up to FVC_NOALLOC_MAX_RAYS pixels;
 * larger ones fail with FVC_ERR_ARG.  `out` holds DEVICE pointers; the work
 * runs on `cuda_stream` (NULL = legacy default stream).  Like fvc_render the
 * call blocks the host: every few sub-iterations it copies the alive-ray
 * count to the host and synchronises the stream, and it returns once the
 * frame has finished marching, so it cannot be called inside a stream
 * capture.  All calls share the scratch:
 * calls whose GPU work overlaps race, so serialise them.  The first call on
 * a device looks the scratch address up (cudaGetSymbolAddress); make it
 * before any stream capture on that device. */
#define FVC_NOALLOC_MAX_RAYS 65536
#define FVC_NOALLOC_SCRATCH_BYTES (48u << 20)
int fvc_render_noalloc(fvc_model *m, const fvc_raymarch_info *info, const fvc_render_outputs *out, void *cuda_stream);

/* ------------------------------------------------------------------------ */
/* frustum volume cache (reference: Cache, include/cache.h:12-74; CacheRenderer */
/* resizeCache / initCacheBlockwise / swapCache / setCacheSettings,             */
/* include/cache_renderer.h:243-267, src/cache_renderer.cu:832-1057)            */
/* ------------------------------------------------------------------------ */
int fvc_cache_create(fvc_cache **out);
void fvc_cache_destroy(fvc_cache *c);
/* Attach the render cache and the build cache ("next") to a cache renderer:
 * CacheRenderer(..., Cache* cache, Cache* next_cache). They may be the same. */
int fvc_renderer_set_caches(fvc_renderer *r, fvc_cache *cache, fvc_cache *next_cache);
/* resizeCache(int2 resolution, StepsizeInfo), src/cache_renderer.cu:832-846. */
int fvc_cache_resize(fvc_renderer *r, int width, int height, const fvc_stepsize_info *steps);

/* The two estimates resizeCache sizes the data array with: samples per ray
 * (INIT_ESTIMATED_N_SAMPLES_PER_RAY, 32) and brick sparsity
 * (INIT_ESTIMATED_BRICK_SPARSITY, 0.5), compile-time constants in the
 * reference (include/cache.h:14-15).  The slots are 128 x 128 x
 * ceil(W H samples / (sparsity 512) / 16384); the next fvc_cache_resize uses
 * them.  A scene whose occupied froxels outnumber the slots overflows (bricks
 * beyond the capacity stay unset and their samples are resampled or dropped,
 * as in the reference). */
int fvc_cache_set_sizing(fvc_renderer *r, int est_samples_per_ray, float brick_sparsity);
/* setCacheSettings, include/cache_renderer.h:75. The settings the cached
 * performance renderer reads (src/cache_performance_renderer.cu:1094,
 * 491, 617, 714): interpol_function for the trilinear weights, and
 * interpol_variant for what a build stores in the voxels' density slot and
 * latent 0 and how a lookup forms the head input. DensityIntermediates
 * needs a model whose first latent is the density, the other variants one
 * whose first latent is not (FVC_ERR_CONFIG at build / render otherwise);
 * Intermediates -> FVC_ERR_CONFIG. The remaining flags only steer the basic
 * cache renderer and are ignored here, as in the reference. */
int fvc_renderer_set_cache_settings(fvc_renderer *r, const fvc_cache_settings *s);
/* initCacheBlockwise(RaymarchInfo, RenderBuffer&), src/cache_renderer.cu:931-1051:
 * fills the "next" cache. Synchronous: returns when the build has finished.
 * It runs on the renderer's lowest-priority stream (the reference's
 * _low_priority_stream) after the work already queued on the renderer's
 * stream, under the write lock, so a build called from another thread
 * overlaps the renders of the current cache (the viewer's double buffering,
 * realtime_viewer/src/application.cu:168-184); fvc_cache_swap then waits for
 * both locks. */
int fvc_cache_build(fvc_renderer *r, const fvc_raymarch_info *info);
/* initCache(RaymarchInfo, RenderBuffer&), src/cache_renderer.cu:848-928: the
 * per-ray fill of the "next" cache (each cache-camera ray marched to its
 * termination, voxels written per visible sample, a ray ending where its
 * brick finds no slot). Slots are reserved per sub-iteration in (brick
 * column, depth) order, not by atomicAdd, so the result is reproducible.
 * Runs on the renderer's render buffers (sized to the cache view) and takes
 * both of its locks. Synchronous; fvc_cache_stats reports n_samples as the
 * reference counts them (padded batches). */
int fvc_cache_build_per_ray(fvc_renderer *r, const fvc_raymarch_info *info);
/* swapCache(), src/cache_renderer.cu:1053-1057. */
int fvc_cache_swap(fvc_renderer *r);
int fvc_cache_stats(fvc_renderer *r, fvc_cache_stats_t *out);
/* Cache render mode (CachePerformanceRenderer::_render_mode). */
int fvc_renderer_set_render_mode(fvc_renderer *r, int mode);

/* Copy cache tables to host for inspection (sizes in elements are returned
 * through *_n when the destination pointer is NULL):
 *   packed_index[bricks]  int32, pack3D(slot) or -1, x fastest
 *                          (Cache::_packed_brick_index_array_3D)
 *   known_ranges[W*H]     float (Cache::_known_ranges_to)
 *   voxels[8*slots*512]   float: density, isset, 0, 0, then 4 words of
 *                          8 fp16 latents, per voxel, slot-major   */
int fvc_cache_read(fvc_cache *c, int32_t *packed_index, size_t *packed_index_n,
                   float *known_ranges, size_t *known_ranges_n,
                   uint32_t *voxels, size_t *voxels_n);
/* Frustum dims (W, H, D), brick dims and data bricks per dim. */
int fvc_cache_dims(fvc_cache *c, fvc_int3 *frustum_dims, fvc_int3 *brick_dims, fvc_int3 *data_bricks_per_dim);

/* ------------------------------------------------------------------------ */
/* batched views (no counterpart in the reference)                           */
/* ------------------------------------------------------------------------ */

/* Plain render of n_views cameras (own resolutions, one shared
 * StepsizeInfo) in one CUDA-graph launch: the sub-iteration loop runs on the
 * device (a conditional WHILE node), with no host round trip per
 * sub-iteration.  Outputs are device buffers holding the views back to back
 * (view v's pixel (x, y) at sum_{u<v} W_u H_u + y * W_v + x).  Asynchronous
 * on the renderer's stream; the graph is rebuilt when the parameters it holds
 * (buffers, counts, path, precision) change. */
int fvc_render_batch(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, const fvc_render_outputs *out);

/* The same for a cache renderer (CACHE_PERFORMANCE): view v renders against
 * its own built frustum cache caches[v] (built with fvc_cache_build after
 * fvc_renderer_set_caches(r, caches[v], caches[v]) at the view's cache pose),
 * as CachePerformanceRenderer::render does for one view. */
int fvc_render_batch_cached(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, fvc_cache *const *caches,
                            const fvc_render_outputs *out);

/* Times each candidate network tile with each compaction batch (rows per
 * sub-iteration: a ray takes clamp(batch / alive rays, 1, 16) samples a
 * sub-iteration, n_steps_curr_subiter of src/performance_renderer.cu:249)
 * and each march length (steps per ray and sub-iteration) on this batch of
 * views, and keeps the fastest for the renderer.  The candidates are those
 * of fvc_renderer_set_autotune_space; by default tcgen05 tiles of 64, 128
 * and 256 rows x batches of 2^16..2^20 rows x march lengths 16 and 64
 * (30 candidates).  No counterpart in the reference (TARGET_BATCH_SIZE is a
 * compile-time constant there). */
typedef struct {
    int m_tile;                  /* rows per network tile of the winner (32: the mma.sync path) */
    int steps_per_iter;          /* marching steps per ray and sub-iteration */
    long long rows_per_iteration;/* mean rows per sub-iteration the winner produced */
    float ms;                    /* its time per batch */
    int n_candidates;
    int batch_rows;              /* the winner's compaction batch */
    int reserved;
} fvc_autotune_result;
int fvc_renderer_autotune(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, const fvc_render_outputs *out,
                          fvc_autotune_result *res);
/* The autotuner's candidate lists (each 1..16 entries): tile heights 64, 128,
 * 256 (tcgen05) or 32 (the mma.sync warp tile); compaction batches in
 * [2^10, 2^26] rows; march lengths, multiples of 4 in [4, 1024]. */
int fvc_renderer_set_autotune_space(fvc_renderer *r, const int *m_tiles, int n_tiles, const int *batch_rows, int n_batches,
                                    const int *march_steps, int n_steps);

/* ------------------------------------------------------------------------ */
/* differentiable render (no counterpart in the reference)                   */
/* ------------------------------------------------------------------------ */

/* Gradients of a model's parameters in fp32, in the model file layouts:
 * hash table [entries x 2] (pos_enc.dat), density MLP blob (mlp_base.dat),
 * color head blob (mlp_head.dat).  Gradients accumulate across
 * fvc_render_backward calls until fvc_grad_zero. */
typedef struct fvc_grad fvc_grad;
int fvc_grad_create(fvc_model *m, fvc_grad **out);
void fvc_grad_destroy(fvc_grad *g);
int fvc_grad_zero(fvc_grad *g);
int fvc_grad_sizes(const fvc_grad *g, size_t *n_table, size_t *n_base, size_t *n_head);
/* copies the accumulated gradients to host arrays (any may be null) */
int fvc_grad_read(fvc_grad *g, float *table, float *base, float *head);
/* gradients of the cache brick latents after cached backward calls: *n =
 * slots x 512 x 8 floats in the cache's [slot][z][y][x][latent] order (0
 * before any cached call); copied to latents when non-null */
int fvc_grad_cache_latents(fvc_grad *g, float *latents, size_t *n);

/* Forward and adjoint of the plain render (renderer kinds BASIC/PERFORMANCE;
 * FP16 or BF16 MLPs per fvc_renderer_set_precision) or of the cached render
 * (CACHE_PERFORMANCE with a built cache, FP16; cache rows also give
 * gradients of the brick latents, fvc_grad_cache_latents)
 * at n_rays pixels (device int32 y * W + x, at most W * H of the camera):
 * L = mean over the rays of sum_k (C_k + T - target_k)^2, the
 * white-background pixel of writeImageBuffer_performance_kernel
 * (src/performance_renderer.cu:127-149) against device target [n_rays x 3].
 * Adds dL/dparam to g, writes L to *loss_out and, if pred is non-null, the
 * forward (C, T) per ray to device pred [n_rays x 4].  The forward is
 * recomputed per sub-iteration instead of stored.  Synchronous. */
int fvc_render_backward(fvc_renderer *r, fvc_grad *g, const fvc_raymarch_info *info, const int32_t *pixels, int n_rays,
                        const float *target, double *loss_out, float *pred);

#ifdef __cplusplus
}
#endif
#endif /* FVC_H */
