/*
 * fvc_capi.cu - host side of the renderer behind the C ABI of include/fvc.h.
 *
 * Owns the model (nerfacc export loader, src/loader.cu:232-300), the
 * renderers (PerformanceRenderer / CachePerformanceRenderer, their
 * resizeRenderbuffers and render), the frustum caches (Cache, CacheRenderer::
 * resizeCache / initCacheBlockwise / swapCache) and their device memory.
 * No exception crosses the ABI: every entry point returns a status and
 * records a thread-local message.
 */
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fvc.h"
#include "fvc_ingp.h"
#include "fvc_kernels.h"

using namespace fvc;

/* The ABI structs have the byte layout of the reference's structs
 * (include/common.h, include/renderer_common.h), measured from those headers. */
static_assert(sizeof(fvc_scene_info) == 76 && offsetof(fvc_scene_info, aabb_from) == 16 &&
              offsetof(fvc_scene_info, contraction_aabb_from) == 40 && offsetof(fvc_scene_info, contraction_type) == 64 &&
              offsetof(fvc_scene_info, is_open_gl) == 68 && offsetof(fvc_scene_info, alpha_thre) == 72, "SceneInfo layout");
static_assert(sizeof(fvc_stepsize_info) == 48, "StepsizeInfo layout");
static_assert(sizeof(fvc_camera_info) == 144 && offsetof(fvc_camera_info, is_open_gl) == 8 && offsetof(fvc_camera_info, focal) == 16 &&
              offsetof(fvc_camera_info, principal) == 24 && offsetof(fvc_camera_info, cam2world) == 32 &&
              offsetof(fvc_camera_info, world2cam) == 80 && offsetof(fvc_camera_info, aperature) == 128 &&
              offsetof(fvc_camera_info, focus_z) == 132, "CameraInfo layout");
static_assert(sizeof(fvc_raymarch_info) == 352 && offsetof(fvc_raymarch_info, next_cam_info) == 144 &&
              offsetof(fvc_raymarch_info, stepsize_info) == 288 && offsetof(fvc_raymarch_info, sample_index) == 336 &&
              offsetof(fvc_raymarch_info, motion_blur) == 340 && offsetof(fvc_raymarch_info, deterministic) == 341, "RaymarchInfo layout");
static_assert(sizeof(fvc_render_stats_t) == 136 && sizeof(fvc_cache_stats_t) == 32, "statistics layout");
static_assert(sizeof(fvc_ray_result) == 16 && sizeof(fvc_camera_matrix) == 48, "BaseRayResult / CameraMatrix layout");

/* ------------------------------------------------------------------------ */
/* errors                                                                    */
/* ------------------------------------------------------------------------ */
static thread_local std::string g_err;

static int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? FVC_ERR_OOM : FVC_ERR_CUDA,              \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    } while (0)

#define CHECK_ARG(cond, msg) \
    do {                     \
        if (!(cond)) return fail(FVC_ERR_ARG, msg); \
    } while (0)

extern "C" const char *fvc_last_error(void) { return g_err.c_str(); }
extern "C" const char *fvc_version(void) { return "fvc-gb300 0.1 (sm_103a)"; }

/* ------------------------------------------------------------------------ */
/* minimal JSON reader (objects, arrays, numbers, strings, bools, null)      */
/* ------------------------------------------------------------------------ */
namespace {
struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    double num = 0;
    bool b = false;
    std::string str;
    std::vector<JVal> arr;
    std::map<std::string, JVal> obj;
    bool has(const std::string &k) const { return kind == OBJ && obj.count(k); }
    const JVal &operator[](const std::string &k) const
    {
        static JVal none;
        auto it = obj.find(k);
        return it == obj.end() ? none : it->second;
    }
    double num_or(const std::string &k, double d) const { return has(k) && (*this)[k].kind == NUM ? (*this)[k].num : d; }
    bool bool_or(const std::string &k, bool d) const { return has(k) && (*this)[k].kind == BOOL ? (*this)[k].b : d; }
};

struct JParser {
    const char *p, *e;
    bool ok = true;
    void ws() { while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p; }
    JVal parse()
    {
        ws();
        JVal v;
        if (p >= e) { ok = false; return v; }
        if (*p == '{') {
            ++p; v.kind = JVal::OBJ; ws();
            if (p < e && *p == '}') { ++p; return v; }
            while (ok) {
                ws();
                JVal k = parse();
                if (k.kind != JVal::STR) { ok = false; break; }
                ws();
                if (p >= e || *p != ':') { ok = false; break; }
                ++p;
                v.obj[k.str] = parse();
                ws();
                if (p < e && *p == ',') { ++p; continue; }
                if (p < e && *p == '}') { ++p; break; }
                ok = false;
            }
        } else if (*p == '[') {
            ++p; v.kind = JVal::ARR; ws();
            if (p < e && *p == ']') { ++p; return v; }
            while (ok) {
                v.arr.push_back(parse());
                ws();
                if (p < e && *p == ',') { ++p; continue; }
                if (p < e && *p == ']') { ++p; break; }
                ok = false;
            }
        } else if (*p == '"') {
            ++p; v.kind = JVal::STR;
            while (p < e && *p != '"') {
                if (*p == '\\' && p + 1 < e) { ++p; v.str.push_back(*p == 'n' ? '\n' : *p); ++p; }
                else v.str.push_back(*p++);
            }
            if (p < e) ++p; else ok = false;
        } else if (!strncmp(p, "true", 4)) { p += 4; v.kind = JVal::BOOL; v.b = true; }
        else if (!strncmp(p, "false", 5)) { p += 5; v.kind = JVal::BOOL; v.b = false; }
        else if (!strncmp(p, "null", 4)) { p += 4; }
        else {
            char *end = nullptr;
            v.num = strtod(p, &end);
            if (end == p) { ok = false; return v; }
            v.kind = JVal::NUM; p = end;
        }
        return v;
    }
};

bool read_file(const std::string &path, std::vector<char> &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    f.seekg(0, std::ios::end);
    out.resize((size_t)f.tellg());
    f.seekg(0);
    f.read(out.data(), (std::streamsize)out.size());
    return (bool)f;
}

/* fp16 bits -> float (exact) */
float h2f(uint16_t h)
{
    const int s = h >> 15, ex = (h >> 10) & 31, m = h & 1023;
    float v;
    if (ex == 0) v = std::ldexp((float)m, -24);
    else if (ex == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((float)(m | 1024), ex - 25);
    return s ? -v : v;
}

/* Pack a row-major [N x K] fp16 matrix into mma.m16n8k16 B fragments:
 * for n-tile j, k-step s, lane (g = lane/4, t = lane%4):
 * b0 = (W[8j+g][16s+2t], W[8j+g][16s+2t+1]), b1 = (.. 16s+2t+8, +9). */
void frag_pack(const std::vector<uint16_t> &W, int N, int K, uint2 *out)
{
    const int KS = K / 16;
    for (int j = 0; j < N / 8; ++j)
        for (int s = 0; s < KS; ++s)
            for (int lane = 0; lane < 32; ++lane) {
                const int g = lane >> 2, t = lane & 3, n = 8 * j + g, k = 16 * s + 2 * t;
                uint2 b;
                b.x = (uint32_t)W[(size_t)n * K + k] | ((uint32_t)W[(size_t)n * K + k + 1] << 16);
                b.y = (uint32_t)W[(size_t)n * K + k + 8] | ((uint32_t)W[(size_t)n * K + k + 9] << 16);
                out[(j * KS + s) * 32 + lane] = b;
            }
}

/* StepsizeInfo::setAdditionalInfo, include/common.h:109-131 (host double),
 * plus the low part of log(1+cone) for fvc_pow_1pc. */
void setup_steps(const fvc_scene_info &sc, fvc_stepsize_info &s)
{
    const float R = 128.0f;
    s.dt_min = s.stepsize;
    s.dt_max = fmaxf(fmaxf((sc.aabb_to.x - sc.aabb_from.x) / R * 1.732f, (sc.aabb_to.y - sc.aabb_from.y) / R * 1.732f),
                     (sc.aabb_to.z - sc.aabb_from.z) / R * 1.732f);
    s.t_min = ((double)s.dt_min) / s.cone_angle;
    const double d_i_min = 1.0 / s.cone_angle;
    s.i_min = d_i_min;
    const double d_log1p_c = std::log(1.0 + s.cone_angle);
    s.log1p_c = d_log1p_c;
    const double d_i_max = std::log(s.dt_max / (double)s.dt_min) / d_log1p_c + d_i_min;
    s.i_max = d_i_max;
    s.t_max = s.t_min * std::pow(1.0 + s.cone_angle, d_i_max - d_i_min);
    /* near_i = step_from_t(near) */
    const float t = s.near_;
    if (s.cone_angle <= 0.0f) s.near_i = t / s.dt_min;
    else if (t >= s.t_max) s.near_i = (t - s.t_max) / s.dt_max + s.i_max;
    else if (t < s.t_min) s.near_i = t / s.dt_min;
    else s.near_i = fvc_logf(t / s.t_min) / s.log1p_c + s.i_min;
}

DevSteps dev_steps(const fvc_stepsize_info &s)
{
    DevSteps d;
    d.cone = s.cone_angle; d.log1p_c = s.log1p_c;
    const double L = std::log(1.0 + (double)s.cone_angle);
    d.log1p_c_lo = (float)(L - (double)s.log1p_c);
    d.near_ = s.near_; d.near_i = s.near_i; d.far_ = s.far_;
    d.dt_min = s.dt_min; d.dt_max = s.dt_max; d.t_min = s.t_min; d.t_max = s.t_max; d.i_min = s.i_min; d.i_max = s.i_max;
    return d;
}

DevCam dev_cam(const fvc_camera_info &c)
{
    DevCam d;
    memset(&d, 0, sizeof(d));
    d.W = c.resolution.x; d.H = c.resolution.y; d.gl = c.is_open_gl ? 1 : 0;
    d.fx = c.focal.x; d.fy = c.focal.y; d.px = c.principal.x; d.py = c.principal.y;
    const fvc_float4 *m = &c.cam2world.m0, *w = &c.world2cam.m0;
    for (int r = 0; r < 3; ++r) {
        d.c2w[4 * r] = m[r].x; d.c2w[4 * r + 1] = m[r].y; d.c2w[4 * r + 2] = m[r].z; d.c2w[4 * r + 3] = m[r].w;
        d.w2c[4 * r] = w[r].x; d.w2c[4 * r + 1] = w[r].y; d.w2c[4 * r + 2] = w[r].z; d.w2c[4 * r + 3] = w[r].w;
    }
    return d;
}

/* the camera with RaymarchInfo's sampling fields (deterministic, motion
 * blur toward next_cam_info, sample index, depth of field) */
DevCam dev_cam_rm(const fvc_raymarch_info &rm)
{
    DevCam d = dev_cam(rm.cam_info);
    d.nd = rm.deterministic ? 0 : 1;
    d.motion_blur = rm.motion_blur ? 1 : 0;
    d.sample_index = rm.sample_index;
    d.aperature = rm.cam_info.aperature;
    d.focus_z = rm.cam_info.focus_z;
    const fvc_float4 *n = &rm.next_cam_info.cam2world.m0;
    for (int r = 0; r < 3; ++r) {
        d.nc2w[4 * r] = n[r].x; d.nc2w[4 * r + 1] = n[r].y; d.nc2w[4 * r + 2] = n[r].z; d.nc2w[4 * r + 3] = n[r].w;
    }
    return d;
}

/* the renderer kinds that render against a frustum cache */
static bool is_cache_kind(int kind) { return kind == FVC_RENDERER_CACHE_PERFORMANCE || kind == FVC_RENDERER_CACHE_BASIC; }

/* fvc_debug_fail_allocation: the library's device allocations still to
 * succeed before one fails (-1: none fails) */
static std::atomic<long long> g_allocs_before_failure{-1};

static bool alloc_failure_due()
{
    long long n = g_allocs_before_failure.load();
    while (n >= 0) {
        if (g_allocs_before_failure.compare_exchange_weak(n, n - 1)) return n == 0;
    }
    return false;
}

template <class T>
int dalloc(T **p, size_t n, const char *what)
{
    *p = nullptr;
    if (n == 0) return FVC_OK;
    if (alloc_failure_due()) return fail(FVC_ERR_OOM, std::string("cudaMalloc ") + what + ": injected allocation failure");
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(FVC_ERR_OOM, std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
    }
    return FVC_OK;
}
template <class T>
void dfree(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}
}  // namespace

/* ------------------------------------------------------------------------ */
/* handles                                                                   */
/* ------------------------------------------------------------------------ */
struct fvc_model {
    int device = 0, n_sms = 0;
    fvc_scene_info scene{};
    fvc_stepsize_info steps{};
    DevScene dscene{};
    DevGrid grid{};
    int latent_offset = 1, n_latents = 8, head_hidden = 2;
    int view_dependent = 0;                 /* split head with an initial view direction (mlp_first_head) */
    int freq = 0;                           /* the head's positional frequency encoding degree (0 or 4) */
    int tc_wbytes = TC_WBYTES;              /* bytes of the tcgen05 weight tiles (TCF_WBYTES with the encoding) */
    std::vector<uint16_t> h_base, h_head;  /* fp16 weight blobs in the model file layouts */
    std::vector<uint16_t> h_first;         /* the first head's blob (view-dependent models) */
    uint8_t *d_weights_vd = nullptr;        /* VD_WBYTES of K-major tiles (view-dependent models) */
    uint2 *d_weights_fh = nullptr;          /* the first head as W_L1 / W_L2 fragment packs */
    uint8_t *d_bits = nullptr;
    __half2 *d_table = nullptr;
    uint2 *d_weights = nullptr;
    uint8_t *d_weights_tc = nullptr;
    uint8_t *d_weights_tc_bf16 = nullptr, *d_weights_tc_fp8 = nullptr;
    float *d_fp8_iw = nullptr;
    float *d_bias3 = nullptr;
    size_t table_entries = 0;
    ~fvc_model()
    {
        dfree(d_bits); dfree(d_table); dfree(d_weights); dfree(d_weights_tc); dfree(d_bias3);
        dfree(d_weights_tc_bf16); dfree(d_weights_tc_fp8); dfree(d_fp8_iw); dfree(d_weights_vd); dfree(d_weights_fh);
    }
};

struct fvc_cache {
    bool initialized = false;
    int fW = 0, fH = 0, fD = 0, bX = 0, bY = 0, bZ = 0, dX = 0, dY = 0, dZ = 0;
    int32_t *d_packed = nullptr;
    float *d_known = nullptr;
    void *d_voxels = nullptr;
    fvc_raymarch_info rm_info{};
    bool built = false;
    fvc_cache_stats_t stats{};
    ~fvc_cache()
    {
        dfree(d_packed); dfree(d_known);
        if (d_voxels) cudaFree(d_voxels);
    }
    int capacity() const { return dX * dY * dZ; }
    CacheView view() const
    {
        CacheView v;
        v.packed_index = d_packed; v.known_ranges = d_known; v.voxels = d_voxels;
        v.fW = fW; v.fH = fH; v.fD = fD; v.bX = bX; v.bY = bY; v.bZ = bZ; v.dX = dX; v.dY = dY; v.dZ = dZ;
        v.n_valid_slots = std::min(stats.n_bricks_demanded, capacity());
        v.interp = 0; v.first_latent_is_density = 0; v.variant = 0; v.reweight = 1; v.keep_first = 1; v.inter_brick = 1;
        return v;
    }
};

struct BuildScratch {
    int n_tiles = 0;
    CacheRay *rays = nullptr;
    int *block_step = nullptr;
    uint8_t *tile_alive = nullptr;
    int *alive_a = nullptr, *alive_b = nullptr;
    int *counters = nullptr;  /* n_alive_a, n_alive_b, slot_counter, n_jobs, guard */
    int *tile_n_samples = nullptr;
    uint8_t *tile_processed = nullptr, *tile_need = nullptr;
    int *tile_n_alive = nullptr;
    int *jobs = nullptr;
    float4 *rows = nullptr;   /* per-iteration sample rows (tiles x 512) */
    __half *den = nullptr;
    uint4 *lat = nullptr;
    int *row_of = nullptr;
    float4 *dirs = nullptr;   /* per-row ray directions (view-dependent models) */
    void release()
    {
        dfree(dirs);
        dfree(rays); dfree(block_step); dfree(tile_alive); dfree(alive_a); dfree(alive_b); dfree(counters);
        dfree(tile_n_samples); dfree(tile_processed); dfree(tile_need); dfree(tile_n_alive); dfree(jobs);
        dfree(rows); dfree(den); dfree(lat); dfree(row_of);
        n_tiles = 0;
    }
};

/* scratch of the per-ray cache fill (fvc_cache_build_per_ray) */
struct PerRayScratch {
    uint8_t *flag = nullptr, *set = nullptr;  /* per brick of the frustum */
    int *col_count = nullptr, *col_base = nullptr;
    int *slots = nullptr;                      /* [0] slot counter, [1] its value before the sub-iteration */
    __half *den = nullptr;                     /* per row */
    uint4 *lat = nullptr;
    size_t n_bricks = 0, n_cols = 0, n_rows = 0;
    void release()
    {
        dfree(flag); dfree(set); dfree(col_count); dfree(col_base); dfree(slots); dfree(den); dfree(lat);
        n_bricks = n_cols = n_rows = 0;
    }
};

struct fvc_renderer {
    fvc_model *m = nullptr;
    int kind = FVC_RENDERER_PERFORMANCE;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t low_prio = nullptr;  /* the blockwise cache build's stream (lowest priority) */
    cudaEvent_t build_after = nullptr; /* orders a build after the work queued on `stream` */
    int W = 0, H = 0;
    int *d_ctl = nullptr;             /* [0] ray counter, [1] guard */
    RenderStatsDev *d_stats = nullptr;
    float4 *d_results = nullptr;
    uchar4 *d_image = nullptr;
    int4 *d_counts = nullptr;
    int *h_pinned = nullptr;          /* readback of build counters */
    /* wavefront buffers (fvc_render.cu) */
    RayState *d_states[2] = {nullptr, nullptr};
    int2 *d_ray_rows = nullptr;
    float *d_row_t0 = nullptr;
    int *d_row_slot = nullptr;
    uint8_t *d_row_kind = nullptr;
    float4 *d_row_pay = nullptr;
    uint4 *d_row_lat = nullptr;
    uint2 *d_row_out = nullptr;
    int *d_res_list = nullptr, *d_cache_list = nullptr;
    int *d_wf_counters = nullptr;
    int row_capacity = 0;
    int last_iterations = 0;
    /* batched views in one graph launch */
    DevCam *d_views = nullptr;
    int *d_view_off = nullptr;
    ViewCache *d_view_caches = nullptr;
    int views_cap = 0;
    cudaGraphExec_t graph_exec = nullptr;
    RenderParams graph_params;        /* the parameters the graph holds by value */
    int graph_head_hidden = 0;
    int graph_kernels = 0;            /* kernels of one loop body + prologue */
    bool last_was_graph = false;
    int steps_per_iter = 64;          /* marching steps per sub-iteration */
    int m_tile = 128;                 /* tcgen05 network tile of the plain path (autotuned) */
    /* the autotuner's candidates (fvc_renderer_set_autotune_space); the default is the batched workload's
     * stated space: tcgen05 tiles {64, 128, 256} x compaction batches 2^16..2^20, march lengths 16 and 64 */
    std::vector<int> tune_tiles{64, 128, 256};
    std::vector<int> tune_batches{1 << 16, 1 << 17, 1 << 18, 1 << 19, 1 << 20};
    std::vector<int> tune_steps{16, 64};
    int row_target = 0;               /* compaction batch, rows per sub-iteration (0: the row capacity; autotuned) */
    int fused_classify = 1;           /* cached renders: classification inside the march (see fvc_renderer_set_fused_classify) */
    int skip_empty = 0;               /* empty-space skipping in the march (fvc_renderer_set_empty_space_skipping); off by
                                       * default: measured slower (the lanes of a warp rarely skip the same steps) */
    int cache_est_samples = 32;       /* cache sizing: estimated samples per ray ... */
    float cache_sparsity = 0.5f;      /* ... and brick sparsity (fvc_cache_set_sizing) */
    float4 *d_row_dout = nullptr;     /* per-row gradients of the differentiable render */
    int *d_grad_rows = nullptr;       /* resample rows with a gradient */
    int *d_grad_cache_rows = nullptr; /* cache rows with a gradient */
    int bwd_capacity = 0;
    LaunchLog log;                    /* kernel accounting of the last render */
    std::vector<cudaEvent_t> events;  /* 2 x 4096 when kernel timing is on */
    void release_wavefront()
    {
        dfree(d_states[0]); dfree(d_states[1]); dfree(d_ray_rows); dfree(d_row_t0); dfree(d_row_slot);
        dfree(d_row_kind); dfree(d_row_pay); dfree(d_row_out); dfree(d_res_list); dfree(d_cache_list); dfree(d_wf_counters);
        dfree(d_row_lat);
        row_capacity = 0;
    }
    fvc_cache *cache = nullptr, *next = nullptr;
    fvc_cache_settings settings{0, 0, 1, 1, 1, 1};
    int render_mode = 0;
    int max_samples = 0;
    int use_tc = 1;                   /* network kernels on tcgen05 (1) or mma.sync (0) */
    int build_tc = 0;                 /* the cache builds' density network on tcgen05 (1) or mma.sync (0, faster) */
    int precision = FVC_PRECISION_FP16;
    BuildScratch bs;
    PerRayScratch pr;
    std::mutex read_mutex, write_mutex;
    ~fvc_renderer()
    {
        if (stream) cudaStreamSynchronize(stream);
        dfree(d_ctl); dfree(d_stats); dfree(d_results); dfree(d_image); dfree(d_counts);
        dfree(d_row_dout); dfree(d_grad_rows); dfree(d_grad_cache_rows);
        dfree(d_views); dfree(d_view_off); dfree(d_view_caches);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        release_wavefront();
        bs.release();
        pr.release();
        if (h_pinned) cudaFreeHost(h_pinned);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        if (own_stream) cudaStreamDestroy(own_stream);
        if (low_prio) cudaStreamDestroy(low_prio);
        if (build_after) cudaEventDestroy(build_after);
    }
};

/* ------------------------------------------------------------------------ */
/* model loading                                                             */
/* ------------------------------------------------------------------------ */
/* The model from its configuration (the nerfacc config.json schema) and its
 * four binary blobs: hash tables, density MLP, color head (fp16) and the
 * linear occupancy grid (uchar [cascade][x][y][z]). */
static int build_model(const JVal &cfg, std::vector<char> &tab, std::vector<char> &wb, std::vector<char> &wh,
                       std::vector<char> &occ, fvc_model &m, const std::vector<char> *wf = nullptr)
{
    const JVal &sc = cfg["scene"];
    if (sc.kind != JVal::OBJ) return fail(FVC_ERR_CONFIG, "config.json: missing scene");
    /* parse(SceneInfo&), include/parse_helper.h:25-54 */
    fvc_scene_info &s = m.scene;
    s.grid_resolution = (int)sc.num_or("grid_resolution", 0);
    s.grid_nlvl = (int)sc.num_or("grid_nlvl", 0);
    s.vals_per_lvl = s.grid_resolution * s.grid_resolution * s.grid_resolution;
    s.normalized = sc.bool_or("normalized", false); /* nerfacc exports: false (include/parse_helper.h:30) */
    if (s.grid_resolution != 128) return fail(FVC_ERR_CONFIG, "Performance Renderer only supports fixed grid resolution!");
    if (s.grid_nlvl < 1 || s.grid_nlvl > 8) return fail(FVC_ERR_CONFIG, "grid_nlvl out of range");
    const JVal &ab = sc["aabb"];
    if (ab.kind != JVal::ARR || ab.arr.size() != 6) return fail(FVC_ERR_CONFIG, "scene.aabb needs 6 values");
    s.aabb_from = {(float)ab.arr[0].num, (float)ab.arr[1].num, (float)ab.arr[2].num};
    s.aabb_to = {(float)ab.arr[3].num, (float)ab.arr[4].num, (float)ab.arr[5].num};
    if (sc.has("contraction") && sc["contraction"].has("aabb")) {
        const JVal &ca = sc["contraction"]["aabb"];
        if (ca.kind != JVal::ARR || ca.arr.size() != 6) return fail(FVC_ERR_CONFIG, "contraction.aabb needs 6 values");
        s.contraction_type = FVC_CONTRACTION_WARP_AABB_LINF;
        s.contraction_aabb_from = {(float)ca.arr[0].num, (float)ca.arr[1].num, (float)ca.arr[2].num};
        s.contraction_aabb_to = {(float)ca.arr[3].num, (float)ca.arr[4].num, (float)ca.arr[5].num};
    } else {
        s.contraction_type = FVC_CONTRACTION_AABB;
    }
    s.is_open_gl = sc.bool_or("is_open_gl", false);
    s.alpha_thre = (float)sc.num_or("alpha_thre", 0.0);
    /* parse(StepsizeInfo&), :57-63 */
    fvc_stepsize_info &st = m.steps;
    st.cone_angle = (float)sc.num_or("cone_angle", 0.0);
    st.stepsize = (float)sc.num_or("stepsize", 0.0);
    st.near_ = (float)sc.num_or("near", 0.0);
    st.far_ = (float)sc.num_or("far", 1e10);
    if (!(st.stepsize > 0.0f)) return fail(FVC_ERR_CONFIG, "scene.stepsize must be > 0");
    setup_steps(s, st);

    /* network */
    const JVal &base = cfg["mlp_base"], &head = cfg["mlp_head"];
    const JVal &enc = base["encoding"];
    const int n_levels = (int)enc.num_or("n_levels", 16), F = (int)enc.num_or("n_features_per_level", 2);
    const int log2T = (int)enc.num_or("log2_hashmap_size", 19), N0 = (int)enc.num_or("base_resolution", 16);
    const float b = (float)enc.num_or("per_level_scale", 2.0);
    if (!((n_levels == 16 && F == 2) || (n_levels == 8 && F == 4)))
        return fail(FVC_ERR_CONFIG, "the hash grid must have 16 levels of 2 features or 8 levels of 4 features");
    if (log2T < 4 || log2T > 24) return fail(FVC_ERR_CONFIG, "log2_hashmap_size out of range");
    const int width = (int)base["network"].num_or("n_neurons", 64);
    if (width != 64 || (int)base["network"].num_or("n_hidden_layers", 1) != 1)
        return fail(FVC_ERR_CONFIG, "density network must be 32 -> 64 -> out (1 hidden layer of 64)");
    const int n_out = (int)base.num_or("n_output", 16);
    if (n_out < 1 || n_out > 16) return fail(FVC_ERR_CONFIG, "mlp_base.n_output must be 1..16");
    /* the view-dependent split network (NerfNetwork::init_viewdep, include/nerf_network.h:120-158,
     * loaded when the config has mlp_first_head, src/loader.cu:251-262): the latents come from a first
     * head on [density outputs | SH of the initial view direction], and the color head reads
     * [latents | SH | SH difference to the initial direction] */
    const JVal &fh = cfg["mlp_first_head"];
    m.view_dependent = fh.kind == JVal::OBJ;
    const bool first_lat_dens = m.view_dependent ? fh.bool_or("first_latent_is_density", true)
                                                 : head.bool_or("first_latent_is_density", true);
    m.latent_offset = first_lat_dens ? 0 : 1;
    m.n_latents = m.view_dependent ? (int)fh.num_or("n_output", 8) : (int)head.num_or("n_latents", n_out);
    /* NerfNetwork::init: freq_encoding_degree (include/nerf_network.h:103); the encoding's 6 * degree values
     * follow the SH inputs of the head (:241-246) */
    m.freq = (int)head.num_or("freq_encoding_degree", 0);
    if (m.freq != 0 && m.freq != 4) return fail(FVC_ERR_CONFIG, "freq_encoding_degree must be 0 or 4");
    const int head_in = (int)head.num_or("n_input", (m.view_dependent ? 32 : 16) + m.n_latents + 6 * m.freq);
    const int head_in_pad = (head_in + 15) / 16 * 16;
    m.head_hidden = (int)head["network"].num_or("n_hidden_layers", 2);
    if ((int)head["network"].num_or("n_neurons", 64) != 64) return fail(FVC_ERR_CONFIG, "head width must be 64");
    if (m.head_hidden < 1 || m.head_hidden > 2) return fail(FVC_ERR_CONFIG, "head must have 1 or 2 hidden layers");
    if (m.view_dependent) {
        if ((int)fh["network"].num_or("n_neurons", 64) != 64 || (int)fh["network"].num_or("n_hidden_layers", 1) != 1)
            return fail(FVC_ERR_CONFIG, "mlp_first_head must be 32 -> 64 -> n_output (1 hidden layer of 64)");
        if (m.n_latents != 8 || m.latent_offset + m.n_latents > 16 || (n_out + 15) / 16 != 1 || (int)fh.num_or("n_input", 32) != 32)
            return fail(FVC_ERR_CONFIG, "mlp_first_head must map the 16 density outputs and 16 SH values to 8 latents");
        if (!m.freq && (head_in != m.n_latents + 32 || head_in_pad != 48))
            return fail(FVC_ERR_CONFIG, "a view-dependent head input must be n_latents + 16 SH + 16 SH differences padded to 48");
        if (m.freq && (head_in != m.n_latents + 32 + 24 || head_in_pad != 64))
            return fail(FVC_ERR_CONFIG, "a view-dependent head with the frequency encoding must read n_latents + 16 SH + 16 SH differences + 24 frequency values (64)");
        const JVal &fn = fh["encoding"]["nested"];
        if (fn.kind == JVal::ARR && fn.arr.size() && (int)fn.arr[0].num_or("degree", 4) != 4)
            return fail(FVC_ERR_CONFIG, "only SH degree 4 direction encoding is built");
        if (!wf) return fail(FVC_ERR_IO, "missing mlp_first_head.dat");
        if (wf->size() != (size_t)(64 * 32 + 16 * 64) * 2) return fail(FVC_ERR_IO, "mlp_first_head.dat has the wrong size");
    } else if (m.freq && (m.latent_offset + m.n_latents > 16 || head_in != m.n_latents + 16 + 24 || head_in_pad != 48)) {
        return fail(FVC_ERR_CONFIG, "a head with the frequency encoding must read n_latents + 16 SH + 24 frequency values (48)");
    } else if (!m.freq && (m.latent_offset + m.n_latents > 16 || head_in != m.n_latents + 16 || head_in_pad != 32)) {
        return fail(FVC_ERR_CONFIG, "head input must be n_latents + 16 SH values padded to 32");
    }
    const JVal &nested = head["encoding"]["nested"];
    if (nested.kind == JVal::ARR && nested.arr.size() && (int)nested.arr[0].num_or("degree", 4) != 4)
        return fail(FVC_ERR_CONFIG, "only SH degree 4 direction encoding is built");

    /* hash-grid levels: scale = N0 * b^l - 1 (float), res = ceil(scale)+1,
     * size = min(round_up(res^3, 8), 2^log2T); explicit fvc_level_scales wins */
    DevGrid &g = m.grid;
    g.n_levels = n_levels;
    g.F = F;
    g.dense_mask = 0;
    const JVal &ls = enc["fvc_level_scales"];
    const float log2b = std::log2(b);
    uint32_t off = 0;
    for (int l = 0; l < n_levels; ++l) {
        float scale = std::exp2((float)l * log2b) * (float)N0 - 1.0f;
        if (ls.kind == JVal::ARR && (int)ls.arr.size() == n_levels) scale = (float)ls.arr[l].num;
        const uint32_t res = (uint32_t)std::ceil(scale) + 1u;
        uint64_t n = (uint64_t)res * res * res;
        n = (n + 7) / 8 * 8;
        const uint32_t size = (uint32_t)std::min<uint64_t>(n, 1ull << log2T);
        g.scale[l] = scale; g.res[l] = res; g.res2[l] = res * res; g.size[l] = size; g.offset[l] = off * (uint32_t)(F / 2);
        if ((uint64_t)res * res * res <= size) g.dense_mask |= 1u << l;
        off += size;
    }
    m.table_entries = off;
    if (tab.size() != (size_t)off * F * 2)
        return fail(FVC_ERR_IO, "pos_enc.dat: " + std::to_string(tab.size()) + " bytes, hash grid needs " + std::to_string((size_t)off * F * 2));
    const int base_out_pad = (n_out + 15) / 16 * 16;
    if (wb.size() != (size_t)(64 * 32 + base_out_pad * 64) * 2) return fail(FVC_ERR_IO, "mlp_base.dat has the wrong size");
    if (wh.size() != (size_t)(64 * head_in_pad + (m.head_hidden - 1) * 64 * 64 + 16 * 64) * 2) return fail(FVC_ERR_IO, "mlp_head.dat has the wrong size");
    const size_t vals = (size_t)128 * 128 * 128;
    if (occ.size() != vals * s.grid_nlvl) return fail(FVC_ERR_IO, "occupancy_grid.dat has the wrong size");

    /* Morton bitfield: occupancy_grid_to_morton_kernel + uchar_to_bitfield
     * (src/loader.cu:20-55) on the host */
    std::vector<uint8_t> bits(vals * s.grid_nlvl / 8, 0);
    auto compact = [](uint32_t x) {
        x &= 0x49249249u; x = (x | (x >> 2)) & 0xc30c30c3u; x = (x | (x >> 4)) & 0x0f00f00fu;
        x = (x | (x >> 8)) & 0xff0000ffu; x = (x | (x >> 16)) & 0x0000ffffu; return x;
    };
    for (size_t i = 0; i < vals * s.grid_nlvl; ++i) {
        const size_t lvl = i / vals;
        const uint32_t j = (uint32_t)(i % vals);
        const uint32_t x = compact(j), y = compact(j >> 1), z = compact(j >> 2);
        if (occ[lvl * vals + (size_t)x * 16384 + y * 128 + z]) bits[i / 8] |= (uint8_t)(1u << (i % 8));
    }

    /* weights -> fragment order */
    auto u16 = [](const std::vector<char> &v, size_t off_h, size_t n) {
        std::vector<uint16_t> o(n);
        memcpy(o.data(), v.data() + off_h * 2, n * 2);
        return o;
    };
    m.h_base = u16(wb, 0, wb.size() / 2);
    m.h_head = u16(wh, 0, wh.size() / 2);
    std::vector<uint2> W(W_TOTAL, make_uint2(0, 0));
    frag_pack(u16(wb, 0, 64 * 32), 64, 32, &W[W_L1]);
    {
        std::vector<uint16_t> w2 = u16(wb, 64 * 32, (size_t)base_out_pad * 64);
        w2.resize(16 * 64, 0);
        frag_pack(w2, 16, 64, &W[W_L2]);
    }
    const int K3 = m.freq ? 64 : 32; /* the kernels' head input: [density outputs 16 | SH 16 (| frequency 24 | 0 8)] */
    std::vector<uint16_t> h0 = u16(wh, 0, (size_t)64 * head_in_pad);
    std::vector<uint16_t> l3((size_t)64 * K3, 0);
    std::vector<float> bias3(64, 0.f);
    /* the head input layout of the kernels; a view-dependent model uses its own tiles (below) instead */
    for (int n = 0; n < 64 && !m.view_dependent; ++n) {
        for (int k = 0; k < 16; ++k) {
            const int src = k - m.latent_offset;
            if (src >= 0 && src < m.n_latents) l3[n * K3 + k] = h0[n * head_in_pad + src];
        }
        for (int j = 0; j < 16; ++j) l3[n * K3 + 16 + j] = h0[n * head_in_pad + m.n_latents + j];
        for (int j = 0; j < 6 * m.freq; ++j) l3[n * K3 + 32 + j] = h0[n * head_in_pad + m.n_latents + 16 + j];
        double acc = 0.0;  /* inputs padded with 1.0 (include/nerf_network.h:248-253) */
        for (int k = head_in; k < head_in_pad; ++k) acc += h2f(h0[n * head_in_pad + k]);
        bias3[n] = (float)acc;
    }
    if (!m.freq) frag_pack(l3, 64, 32, &W[W_L3]); /* the mma.sync path has no frequency encoding */
    size_t ho = (size_t)64 * head_in_pad;
    const size_t h_l4 = ho; /* the second hidden layer's weights */
    if (m.head_hidden == 2) {
        frag_pack(u16(wh, ho, 64 * 64), 64, 64, &W[W_L4]);
        ho += 64 * 64;
    }
    frag_pack(u16(wh, ho, 16 * 64), 16, 64, &W[W_L5]);

    /* the same matrices as canonical K-major tiles for the tcgen05 kernels (the head's first layer with
     * K = 64 and the later layers shifted for a frequency-encoded head) */
    m.tc_wbytes = m.freq ? TCF_WBYTES : TC_WBYTES;
    std::vector<uint8_t> Wt(m.tc_wbytes, 0);
    auto tc_pack = [&](const std::vector<uint16_t> &M, int N, int K, int off) {
        for (int n = 0; n < N; ++n)
            for (int k = 0; k < K; ++k) memcpy(&Wt[off + kmajor_offset(n, k, K)], &M[(size_t)n * K + k], 2);
    };
    tc_pack(u16(wb, 0, 64 * 32), 64, 32, TC_B1);
    {
        std::vector<uint16_t> w2 = u16(wb, 64 * 32, (size_t)base_out_pad * 64);
        w2.resize(16 * 64, 0);
        tc_pack(w2, 16, 64, TC_B2);
    }
    tc_pack(l3, 64, K3, m.freq ? TCF_B3 : TC_B3);
    if (m.head_hidden == 2) tc_pack(u16(wh, h_l4, 64 * 64), 64, 64, m.freq ? TCF_B4 : TC_B4);
    tc_pack(u16(wh, ho, 16 * 64), 16, 64, m.freq ? TCF_B5 : TC_B5);

    /* reduced-precision copies: bf16 tiles (same layout) and e4m3 tiles
     * (8-bit K-major layout), each e4m3 layer scaled by 448 / amax(W); none for a frequency-encoded head */
    if (!m.freq) {
        std::vector<uint8_t> Wb(TC_WBYTES, 0), W8(TC8_WBYTES, 0);
        float iw[5] = {1.f, 1.f, 1.f, 1.f, 1.f};
        auto pack_low = [&](const std::vector<uint16_t> &M, int N, int K, int off16, int off8, int layer) {
            float amax = 0.f;
            for (uint16_t h : M) amax = std::max(amax, std::fabs(h2f(h)));
            const float sc = amax > 0.f ? 448.0f / amax : 1.0f;
            iw[layer] = 1.0f / sc;
            for (int n = 0; n < N; ++n)
                for (int k = 0; k < K; ++k) {
                    const float v = h2f(M[(size_t)n * K + k]);
                    const __nv_bfloat16 b = __float2bfloat16_rn(v);
                    memcpy(&Wb[off16 + kmajor_offset(n, k, K)], &b, 2);
                    W8[off8 + kmajor_offset8(n, k, K)] = (uint8_t)__nv_cvt_float_to_fp8(v * sc, __NV_SATFINITE, __NV_E4M3);
                }
        };
        pack_low(u16(wb, 0, 64 * 32), 64, 32, TC_B1, TC8_B1, 0);
        std::vector<uint16_t> w2 = u16(wb, 64 * 32, (size_t)base_out_pad * 64);
        w2.resize(16 * 64, 0);
        pack_low(w2, 16, 64, TC_B2, TC8_B2, 1);
        pack_low(l3, 64, 32, TC_B3, TC8_B3, 2);
        if (m.head_hidden == 2) pack_low(u16(wh, 64 * 32, 64 * 64), 64, 64, TC_B4, TC8_B4, 3);
        pack_low(u16(wh, ho, 16 * 64), 16, 64, TC_B5, TC8_B5, 4);
        int rc;
        if ((rc = dalloc(&m.d_weights_tc_bf16, (size_t)TC_WBYTES, "bf16 weights"))) return rc;
        if ((rc = dalloc(&m.d_weights_tc_fp8, (size_t)TC8_WBYTES, "fp8 weights"))) return rc;
        if ((rc = dalloc(&m.d_fp8_iw, (size_t)8, "fp8 scales"))) return rc;
        CU(cudaMemcpy(m.d_weights_tc_bf16, Wb.data(), TC_WBYTES, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(m.d_weights_tc_fp8, W8.data(), TC8_WBYTES, cudaMemcpyHostToDevice));
        CU(cudaMemcpy(m.d_fp8_iw, iw, sizeof(iw), cudaMemcpyHostToDevice));
    }

    /* the view-dependent network: the first head as fragment packs (the cache build's density kernel)
     * and every layer as K-major tiles (the tcgen05 network kernel); its color head keeps the model's
     * input order and reads the 1-padding through its weights */
    if (m.view_dependent) {
        m.h_first = u16(*wf, 0, wf->size() / 2);
        std::vector<uint2> Wf(W_L3, make_uint2(0, 0));
        frag_pack(u16(*wf, 0, 64 * 32), 64, 32, &Wf[W_L1]);
        frag_pack(u16(*wf, 64 * 32, 16 * 64), 16, 64, &Wf[W_L2]);
        const int vd_bytes = m.freq ? VDF_WBYTES : VD_WBYTES;
        std::vector<uint8_t> Wv(vd_bytes, 0);
        auto vd_pack = [&](const std::vector<uint16_t> &M, int N, int K, int off) {
            for (int n = 0; n < N; ++n)
                for (int k = 0; k < K; ++k) memcpy(&Wv[off + kmajor_offset(n, k, K)], &M[(size_t)n * K + k], 2);
        };
        vd_pack(u16(wb, 0, 64 * 32), 64, 32, VD_B1);
        std::vector<uint16_t> w2 = u16(wb, 64 * 32, (size_t)base_out_pad * 64);
        w2.resize(16 * 64, 0);
        vd_pack(w2, 16, 64, VD_B2);
        vd_pack(u16(*wf, 0, 64 * 32), 64, 32, VD_F1);
        vd_pack(u16(*wf, 64 * 32, 16 * 64), 16, 64, VD_F2);
        vd_pack(u16(wh, 0, (size_t)64 * head_in_pad), 64, head_in_pad, VD_B3);
        size_t vo = (size_t)64 * head_in_pad;
        if (m.head_hidden == 2) {
            vd_pack(u16(wh, vo, 64 * 64), 64, 64, m.freq ? VDF_B4 : VD_B4);
            vo += 64 * 64;
        }
        vd_pack(u16(wh, vo, 16 * 64), 16, 64, m.freq ? VDF_B5 : VD_B5);
        int rc;
        if ((rc = dalloc(&m.d_weights_fh, Wf.size(), "first-head weights"))) return rc;
        if ((rc = dalloc(&m.d_weights_vd, (size_t)vd_bytes, "view-dependent weights"))) return rc;
        CU(cudaMemcpy(m.d_weights_fh, Wf.data(), Wf.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(m.d_weights_vd, Wv.data(), vd_bytes, cudaMemcpyHostToDevice));
    }

    /* device scene block */
    DevScene &d = m.dscene;
    d.aabb_from = make_float3(s.aabb_from.x, s.aabb_from.y, s.aabb_from.z);
    d.aabb_to = make_float3(s.aabb_to.x, s.aabb_to.y, s.aabb_to.z);
    const float sc2 = (float)(1 << (s.grid_nlvl - 1));
    d.unit_off = make_float3(s.aabb_from.x / sc2, s.aabb_from.y / sc2, s.aabb_from.z / sc2);
    d.unit_den = make_float3((s.aabb_to.x - s.aabb_from.x) / sc2, (s.aabb_to.y - s.aabb_from.y) / sc2, (s.aabb_to.z - s.aabb_from.z) / sc2);
    d.aabb_den = make_float3(s.aabb_to.x - s.aabb_from.x, s.aabb_to.y - s.aabb_from.y, s.aabb_to.z - s.aabb_from.z);
    /* correctly rounded reciprocals for the kernels' exact divisions (div_rn_by) */
    d.unit_rcp = make_float3(1.0f / d.unit_den.x, 1.0f / d.unit_den.y, 1.0f / d.unit_den.z);
    d.aabb_rcp = make_float3(1.0f / d.aabb_den.x, 1.0f / d.aabb_den.y, 1.0f / d.aabb_den.z);
    d.c_from = make_float3(s.contraction_aabb_from.x, s.contraction_aabb_from.y, s.contraction_aabb_from.z);
    d.c_den = make_float3(s.contraction_aabb_to.x - s.contraction_aabb_from.x, s.contraction_aabb_to.y - s.contraction_aabb_from.y,
                          s.contraction_aabb_to.z - s.contraction_aabb_from.z);
    d.c_rcp = make_float3(1.0f / d.c_den.x, 1.0f / d.c_den.y, 1.0f / d.c_den.z);
    d.nlvl = s.grid_nlvl; d.normalized = s.normalized; d.contraction = s.contraction_type; d.is_open_gl = s.is_open_gl;
    d.alpha_thre = s.alpha_thre;

    CU(cudaGetDevice(&m.device));
    CU(cudaDeviceGetAttribute(&m.n_sms, cudaDevAttrMultiProcessorCount, m.device));
    int rc;
    if ((rc = dalloc(&m.d_bits, bits.size(), "occupancy bits"))) return rc;
    if ((rc = dalloc(&m.d_table, (size_t)off * (F / 2), "hash tables"))) return rc;
    if ((rc = dalloc(&m.d_weights, (size_t)W_TOTAL, "weights"))) return rc;
    if ((rc = dalloc(&m.d_bias3, (size_t)64, "bias"))) return rc;
    if ((rc = dalloc(&m.d_weights_tc, (size_t)m.tc_wbytes, "tcgen05 weights"))) return rc;
    CU(cudaMemcpy(m.d_weights_tc, Wt.data(), m.tc_wbytes, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(m.d_bits, bits.data(), bits.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(m.d_table, tab.data(), tab.size(), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(m.d_weights, W.data(), W.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    CU(cudaMemcpy(m.d_bias3, bias3.data(), 64 * sizeof(float), cudaMemcpyHostToDevice));
    return FVC_OK;
}

/* load_nerfacc_export (src/loader.cu:232-285): config.json and four blobs */
static int load_nerfacc(const std::string &dir, fvc_model &m)
{
    std::vector<char> txt, tab, wb, wh, occ;
    if (!read_file(dir + "/config.json", txt)) return fail(FVC_ERR_IO, "Could not load config file: " + dir + "/config.json");
    JParser jp{txt.data(), txt.data() + txt.size()};
    JVal cfg = jp.parse();
    if (!jp.ok || cfg.kind != JVal::OBJ) return fail(FVC_ERR_CONFIG, "config.json: parse error");
    if (!read_file(dir + "/pos_enc.dat", tab)) return fail(FVC_ERR_IO, "missing pos_enc.dat");
    if (!read_file(dir + "/mlp_base.dat", wb)) return fail(FVC_ERR_IO, "missing mlp_base.dat");
    if (!read_file(dir + "/mlp_head.dat", wh)) return fail(FVC_ERR_IO, "missing mlp_head.dat");
    if (!read_file(dir + "/occupancy_grid.dat", occ)) return fail(FVC_ERR_IO, "missing occupancy_grid.dat");
    std::vector<char> wf;
    const bool vd = cfg["mlp_first_head"].kind == JVal::OBJ;
    if (vd && !read_file(dir + "/mlp_first_head.dat", wf)) return fail(FVC_ERR_IO, "missing mlp_first_head.dat");
    return build_model(cfg, tab, wb, wh, occ, m, vd ? &wf : nullptr);
}

/* load_ingp_snapshot (src/loader.cu:146-230): the scene, step grid and
 * network configuration the reference derives from an instant-ngp snapshot,
 * the parameter blob split in its set_params order (density MLP, color MLP,
 * hash grid; include/nerf_network.h:284-298), and the occupancy grid from the
 * density grid thresholded at min(0.01, mean density of the first cascade)
 * (ingp_density_grid_to_occupancy_grid, :73-114; the mean in float64). */
static int ingp_to_export(const std::string &file, JVal &cfg, std::vector<char> &tab, std::vector<char> &wb,
                          std::vector<char> &wh, std::vector<char> &occ)
{
    fvc_ingp::Snapshot sn;
    std::string err;
    if (!fvc_ingp::read_snapshot(file, sn, err)) return fail(FVC_ERR_IO, err);
    auto num = [](double v) { JVal j; j.kind = JVal::NUM; j.num = v; return j; };
    auto flag = [](bool v) { JVal j; j.kind = JVal::BOOL; j.b = v; return j; };
    auto obj = []() { JVal j; j.kind = JVal::OBJ; return j; };
    if (sn.aabb_scale < 1 || (sn.aabb_scale & (sn.aabb_scale - 1))) return fail(FVC_ERR_CONFIG, "aabb_scale must be a power of two");
    const int nlvl = (int)std::log2((double)sn.aabb_scale) + 1;
    JVal scene = obj();
    scene.obj["grid_resolution"] = num(128);
    scene.obj["grid_nlvl"] = num(nlvl);
    scene.obj["normalized"] = flag(true);
    JVal aabb;
    aabb.kind = JVal::ARR;
    for (int k = 0; k < 3; ++k) aabb.arr.push_back(num(sn.aabb_min[k]));
    for (int k = 0; k < 3; ++k) aabb.arr.push_back(num(sn.aabb_max[k]));
    scene.obj["aabb"] = aabb;
    scene.obj["is_open_gl"] = flag(false);
    scene.obj["alpha_thre"] = num(0.0);
    scene.obj["cone_angle"] = num(nlvl <= 1 ? 0.0f : 1.0f / 256.0f);
    scene.obj["stepsize"] = num(std::sqrt(3.0f) / 1024.f);
    scene.obj["near"] = num(0.0);
    scene.obj["far"] = num(1e10f);
    JVal enc = obj();
    enc.obj["n_levels"] = num(sn.n_levels);
    enc.obj["n_features_per_level"] = num(sn.n_features);
    enc.obj["log2_hashmap_size"] = num(sn.log2_hashmap_size);
    enc.obj["base_resolution"] = num(sn.base_resolution);
    const float pls = std::exp(std::log(2048.f * (float)sn.aabb_scale / (float)sn.base_resolution) / (float)(sn.n_levels - 1.f));
    enc.obj["per_level_scale"] = num(pls);
    JVal bnet = obj(), hnet = obj();
    bnet.obj["n_neurons"] = num(sn.base_neurons);
    bnet.obj["n_hidden_layers"] = num(sn.base_hidden);
    hnet.obj["n_neurons"] = num(sn.head_neurons);
    hnet.obj["n_hidden_layers"] = num(sn.head_hidden);
    JVal base = obj(), head = obj();
    base.obj["encoding"] = enc;
    base.obj["network"] = bnet;
    base.obj["n_output"] = num(16);
    head.obj["network"] = hnet;
    head.obj["first_latent_is_density"] = flag(true); /* NerfNetwork::init keeps the default */
    head.obj["n_latents"] = num(16);
    head.obj["n_input"] = num(32);
    JVal nested;
    nested.kind = JVal::ARR;
    JVal sh = obj();
    sh.obj["degree"] = num(sn.sh_degree);
    nested.arr.push_back(sh);
    JVal dir_enc = obj();
    dir_enc.obj["nested"] = nested;
    head.obj["encoding"] = dir_enc;
    cfg = obj();
    cfg.obj["scene"] = scene;
    cfg.obj["mlp_base"] = base;
    cfg.obj["mlp_head"] = head;
    /* parameter blob: density MLP [64 x 32][16 x 64], color MLP [64 x 32]([64 x 64])[16 x 64], hash grid */
    const size_t n_base = 64 * 32 + 16 * 64;
    const size_t n_head = 64 * 32 + (size_t)std::max(0, sn.head_hidden - 1) * 64 * 64 + 16 * 64;
    if (sn.params.size() < n_base + n_head) return fail(FVC_ERR_IO, file + ": params_binary too small for the networks");
    auto bytes = [&](size_t off, size_t n) {
        std::vector<char> v(n * 2);
        std::memcpy(v.data(), sn.params.data() + off, n * 2);
        return v;
    };
    wb = bytes(0, n_base);
    wh = bytes(n_base, n_head);
    tab = bytes(n_base + n_head, sn.params.size() - n_base - n_head);
    /* occupancy: density grid (Morton order per cascade) -> linear uchar [cascade][x][y][z] */
    const size_t vals = (size_t)128 * 128 * 128;
    if (sn.density_grid.size() != vals * nlvl) return fail(FVC_ERR_IO, file + ": density_grid_binary does not hold the cascades");
    double mean = 0.0;
    for (size_t i = 0; i < vals; ++i) mean += std::max(0.0f, h2f(sn.density_grid[i])) / (double)vals;
    const float thresh = std::min(0.01f, (float)mean);
    auto compact = [](uint32_t x) {
        x &= 0x49249249u; x = (x | (x >> 2)) & 0xc30c30c3u; x = (x | (x >> 4)) & 0x0f00f00fu;
        x = (x | (x >> 8)) & 0xff0000ffu; x = (x | (x >> 16)) & 0x0000ffffu; return x;
    };
    occ.assign(vals * nlvl, 0);
    for (size_t i = 0; i < vals * nlvl; ++i) {
        const size_t lvl = i / vals;
        const uint32_t j = (uint32_t)(i % vals);
        const uint32_t x = compact(j), y = compact(j >> 1), z = compact(j >> 2);
        occ[lvl * vals + (size_t)x * 16384 + y * 128 + z] = h2f(sn.density_grid[i]) > thresh ? 1 : 0;
    }
    return FVC_OK;
}

static int load_ingp(const std::string &file, fvc_model &m)
{
    JVal cfg;
    std::vector<char> tab, wb, wh, occ;
    if (int rc = ingp_to_export(file, cfg, tab, wb, wh, occ)) return rc;
    return build_model(cfg, tab, wb, wh, occ, m);
}

static void write_json(const JVal &v, std::string &o)
{
    char buf[40];
    switch (v.kind) {
        case JVal::NUL: o += "null"; break;
        case JVal::BOOL: o += v.b ? "true" : "false"; break;
        case JVal::NUM: std::snprintf(buf, sizeof buf, "%.17g", v.num); o += buf; break;
        case JVal::STR: o += '"' + v.str + '"'; break;
        case JVal::ARR:
            o += '[';
            for (size_t i = 0; i < v.arr.size(); ++i) {
                if (i) o += ", ";
                write_json(v.arr[i], o);
            }
            o += ']';
            break;
        case JVal::OBJ: {
            o += '{';
            bool first = true;
            for (const auto &kv : v.obj) {
                if (!first) o += ", ";
                first = false;
                o += '"' + kv.first + "\": ";
                write_json(kv.second, o);
            }
            o += '}';
            break;
        }
    }
}

static bool write_blob(const std::string &path, const std::string &data)
{
    std::ofstream f(path, std::ios::binary);
    f.write(data.data(), (std::streamsize)data.size());
    return (bool)f;
}

/* load_data (src/loader.cu:287-300): an .ingp snapshot file or a nerfacc export directory */
static bool is_ingp(const std::string &path) { return std::filesystem::path(path).extension() == ".ingp"; }

static int load_model(const std::string &path, fvc_model &m)
{
    return is_ingp(path) ? load_ingp(path, m) : load_nerfacc(path, m);
}

/* host only: an .ingp snapshot rewritten as the equivalent nerfacc export */
extern "C" int fvc_ingp_export(const char *snapshot, const char *export_dir)
{
    CHECK_ARG(snapshot && export_dir, "fvc_ingp_export: null argument");
    JVal cfg;
    std::vector<char> tab, wb, wh, occ;
    if (int rc = ingp_to_export(snapshot, cfg, tab, wb, wh, occ)) return rc;
    std::error_code ec;
    std::filesystem::create_directories(export_dir, ec);
    const std::string dir(export_dir);
    std::string js;
    write_json(cfg, js);
    auto str = [](const std::vector<char> &v) { return std::string(v.data(), v.size()); };
    if (!write_blob(dir + "/config.json", js) || !write_blob(dir + "/pos_enc.dat", str(tab)) ||
        !write_blob(dir + "/mlp_base.dat", str(wb)) || !write_blob(dir + "/mlp_head.dat", str(wh)) ||
        !write_blob(dir + "/occupancy_grid.dat", str(occ)))
        return fail(FVC_ERR_IO, "fvc_ingp_export: could not write " + dir);
    return FVC_OK;
}

/* the head's tcgen05 tile layout of a model (TC_* without, TCF_* with the frequency encoding) */
static void set_head_layout(const fvc_model &m, RenderParams &p)
{
    p.freq = m.freq;
}

extern "C" int fvc_model_load(const char *data_dir, fvc_model **out)
{
    CHECK_ARG(data_dir && out, "fvc_model_load: null argument");
    *out = nullptr;
    auto m = std::make_unique<fvc_model>();
    const int rc = load_model(data_dir, *m);
    if (rc) return rc;
    *out = m.release();
    return FVC_OK;
}

extern "C" void fvc_model_destroy(fvc_model *m) { delete m; }

extern "C" int fvc_model_info(const fvc_model *m, fvc_scene_info *scene, fvc_stepsize_info *steps)
{
    CHECK_ARG(m, "fvc_model_info: null model");
    if (scene) *scene = m->scene;
    if (steps) *steps = m->steps;
    return FVC_OK;
}

extern "C" int fvc_debug_fail_allocation(long long n)
{
    CHECK_ARG(n >= -1, "fvc_debug_fail_allocation: n must be >= -1");
    g_allocs_before_failure.store(n);
    return FVC_OK;
}

extern "C" int fvc_selftest_wait_timeout(double limit_ms, double *waited_ms)
{
    CHECK_ARG(limit_ms > 0.0 && limit_ms <= 1000.0, "fvc_selftest_wait_timeout: limit must be in (0, 1000] ms");
    int dev = 0, khz = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
    long long *d = nullptr;
    int rc;
    if ((rc = dalloc(&d, (size_t)2, "wait self-test"))) return rc;
    long long h[2] = {0, 0};
    const long long limit = (long long)(limit_ms * (double)khz);
    cudaError_t e = launch_wait_selftest(limit, d, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    dfree(d);
    if (e != cudaSuccess) return fail(FVC_ERR_CUDA, std::string("wait self-test: ") + cudaGetErrorString(e));
    if (waited_ms) *waited_ms = (double)h[1] / (double)khz;
    if (h[0]) return fail(FVC_ERR_TIMEOUT, "bounded device wait gave up after " + std::to_string((double)h[1] / khz) + " ms");
    return FVC_OK;
}

extern "C" int fvc_selftest_division(const float *x, const float *d, int n, float *q, float *q_ieee)
{
    CHECK_ARG(x && d && q && q_ieee && n > 0 && n <= (1 << 24), "fvc_selftest_division: bad arguments");
    float *b = nullptr;
    int rc;
    if ((rc = dalloc(&b, (size_t)4 * n, "division self-test"))) return rc;
    cudaError_t e = cudaMemcpy(b, x, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b + n, d, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_div_selftest(b, b + n, n, b + 2 * (size_t)n, b + 3 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(q, b + 2 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(q_ieee, b + 3 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost);
    dfree(b);
    if (e != cudaSuccess) return fail(FVC_ERR_CUDA, std::string("division self-test: ") + cudaGetErrorString(e));
    return FVC_OK;
}

extern "C" int fvc_stepsize_setup(const fvc_scene_info *scene, fvc_stepsize_info *steps)
{
    CHECK_ARG(scene && steps, "fvc_stepsize_setup: null argument");
    CHECK_ARG(steps->stepsize > 0.0f && steps->cone_angle >= 0.0f, "fvc_stepsize_setup: stepsize must be > 0, cone_angle >= 0");
    setup_steps(*scene, *steps);
    return FVC_OK;
}

static int run_inference(fvc_model *m, const float *pos, const float *dir, int n, float *out4, float *base_out, float *features)
{
    CHECK_ARG(m && pos && n >= 0, "inference: bad arguments");
    if (m->freq && dir) return fail(FVC_ERR_CONFIG, "network inference evaluates heads without the frequency encoding");
    if (n == 0) return FVC_OK;
    float *dp = nullptr, *dd = nullptr, *d4 = nullptr, *db = nullptr, *df = nullptr;
    int rc = FVC_OK;
    struct Guard {
        float **p[5];
        ~Guard() { for (auto q : p) dfree(*q); }
    } guard{{&dp, &dd, &d4, &db, &df}};
    if ((rc = dalloc(&dp, (size_t)3 * n, "inference input"))) return rc;
    if (dir && (rc = dalloc(&dd, (size_t)3 * n, "inference dir"))) return rc;
    if (out4 && (rc = dalloc(&d4, (size_t)4 * n, "inference out"))) return rc;
    if (base_out && (rc = dalloc(&db, (size_t)16 * n, "inference base"))) return rc;
    if (features && (rc = dalloc(&df, (size_t)32 * n, "inference features"))) return rc;
    CU(cudaMemcpy(dp, pos, sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
    if (dir) CU(cudaMemcpy(dd, dir, sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
    InferenceParams p;
    p.grid = m->grid; p.table = m->d_table; p.weights = m->d_weights; p.bias3 = m->d_bias3;
    p.pos = dp; p.dir = dd; p.n = n; p.out4 = d4; p.base_out = db; p.features = df;
    CU(launch_inference(p, m->head_hidden, m->n_sms, 0));
    CU(cudaDeviceSynchronize());
    if (out4) CU(cudaMemcpy(out4, d4, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost));
    if (base_out) CU(cudaMemcpy(base_out, db, sizeof(float) * 16 * n, cudaMemcpyDeviceToHost));
    if (features) CU(cudaMemcpy(features, df, sizeof(float) * 32 * n, cudaMemcpyDeviceToHost));
    return FVC_OK;
}

extern "C" int fvc_model_density(fvc_model *m, const float *pos, int n, float *log_density_out)
{
    std::vector<float> o4((size_t)4 * n);
    const int rc = run_inference(m, pos, nullptr, n, o4.data(), nullptr, nullptr);
    if (rc) return rc;
    for (int i = 0; i < n; ++i) log_density_out[i] = o4[(size_t)4 * i + 3];
    return FVC_OK;
}

extern "C" int fvc_model_inference(fvc_model *m, const float *pos, const float *dir01, int n, float *out)
{
    CHECK_ARG(m && dir01 && out, "fvc_model_inference: null argument");
    if (m->view_dependent) return fail(FVC_ERR_CONFIG, "view-dependent models (mlp_first_head) are built for the renderers and cache builds on the tcgen05 network path in FP16 (the autotuner also tries the mma.sync path)");
    return run_inference(m, pos, dir01, n, out, nullptr, nullptr);
}

/* test hook: hash features and density-network outputs at given positions */
extern "C" int fvc_model_debug_encode(fvc_model *m, const float *pos, int n, float *features32, float *base_out16)
{
    return run_inference(m, pos, nullptr, n, nullptr, base_out16, features32);
}

/* ------------------------------------------------------------------------ */
/* renderers                                                                 */
/* ------------------------------------------------------------------------ */
extern "C" int fvc_renderer_create(fvc_model *m, int kind, fvc_renderer **out)
{
    CHECK_ARG(m && out, "fvc_renderer_create: null argument");
    CHECK_ARG(kind >= FVC_RENDERER_BASIC && kind <= FVC_RENDERER_CACHE_BASIC, "fvc_renderer_create: unknown kind");
    *out = nullptr;
    auto r = std::make_unique<fvc_renderer>();
    r->m = m;
    r->kind = kind;
    CU(cudaStreamCreateWithFlags(&r->own_stream, cudaStreamNonBlocking));
    r->stream = r->own_stream;
    int lo = 0, hi = 0;
    CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CU(cudaStreamCreateWithPriority(&r->low_prio, cudaStreamNonBlocking, lo)); /* src/cache_renderer.cu:822-825 */
    CU(cudaEventCreateWithFlags(&r->build_after, cudaEventDisableTiming));
    int rc;
    if ((rc = dalloc(&r->d_ctl, (size_t)4, "control words"))) return rc;
    if ((rc = dalloc(&r->d_stats, (size_t)1, "stats"))) return rc;
    CU(cudaMallocHost((void **)&r->h_pinned, 16 * sizeof(int)));
    CU(cudaMemset(r->d_stats, 0, sizeof(RenderStatsDev)));
    CU(cudaMemset(r->d_ctl, 0, 4 * sizeof(int)));
    *out = r.release();
    return FVC_OK;
}

extern "C" void fvc_renderer_destroy(fvc_renderer *r) { delete r; }

extern "C" int fvc_renderer_set_stream(fvc_renderer *r, void *s)
{
    CHECK_ARG(r, "fvc_renderer_set_stream: null renderer");
    r->stream = s ? (cudaStream_t)s : r->own_stream;
    return FVC_OK;
}

extern "C" int fvc_renderer_resize(fvc_renderer *r, int width, int height)
{
    CHECK_ARG(r && width > 0 && height > 0, "fvc_renderer_resize: bad arguments");
    if (width == r->W && height == r->H) return FVC_OK;
    CU(cudaStreamSynchronize(r->stream));
    dfree(r->d_results); dfree(r->d_image); dfree(r->d_counts);
    const size_t n = (size_t)width * height;
    int rc;
    if ((rc = dalloc(&r->d_results, n, "results"))) return rc;
    if ((rc = dalloc(&r->d_image, n, "image"))) return rc;
    if ((rc = dalloc(&r->d_counts, n, "ray counts"))) return rc;
    CU(cudaMemset(r->d_image, 0, n * sizeof(uchar4)));
    /* wavefront: alive-ray states (ping-pong) and up to 16 sample rows per
     * ray and sub-iteration */
    r->release_wavefront();
    /* at least one row per ray: the march gives each alive ray
     * min(16, capacity / alive) rows, so capacity >= rays keeps that >= 1 */
    const size_t cap = std::max(n, std::min<size_t>(n * 16, (size_t)1 << 25));
    const bool cached = is_cache_kind(r->kind);
    if ((rc = dalloc(&r->d_states[0], n, "ray states"))) return rc;
    if ((rc = dalloc(&r->d_states[1], n, "ray states"))) return rc;
    if ((rc = dalloc(&r->d_ray_rows, n, "ray rows"))) return rc;
    if ((rc = dalloc(&r->d_row_t0, cap, "row t0"))) return rc;
    if ((rc = dalloc(&r->d_row_slot, cap, "row slots"))) return rc;
    if ((rc = dalloc(&r->d_row_pay, cap, "row inputs"))) return rc;
    if ((rc = dalloc(&r->d_row_out, cap, "row outputs"))) return rc;
    if (cached) {
        if ((rc = dalloc(&r->d_row_kind, cap, "row kinds"))) return rc;
        if ((rc = dalloc(&r->d_res_list, cap, "resample list"))) return rc;
        if ((rc = dalloc(&r->d_cache_list, cap, "cache list"))) return rc;
        if ((rc = dalloc(&r->d_row_lat, cap, "cache-row head inputs"))) return rc;
    }
    if ((rc = dalloc(&r->d_wf_counters, (size_t)8, "wavefront counters"))) return rc;
    r->row_capacity = (int)cap;
    r->W = width; r->H = height;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_max_samples_per_ray(fvc_renderer *r, int n)
{
    CHECK_ARG(r && n >= 0, "fvc_renderer_set_max_samples_per_ray: bad arguments");
    r->max_samples = n;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_render_mode(fvc_renderer *r, int mode)
{
    CHECK_ARG(r && mode >= 0 && mode <= 2, "fvc_renderer_set_render_mode: bad mode");
    r->render_mode = mode;
    return FVC_OK;
}

static int check_info(const fvc_raymarch_info *info, bool cache_build = false)
{
    if (cache_build && !info->deterministic)
        return fail(FVC_ERR_CONFIG, "cache builds march the pixel centres: RaymarchInfo::deterministic must be true");
    if (!info->deterministic && info->cam_info.aperature != 0.0f && !(info->cam_info.focus_z != 0.0f))
        return fail(FVC_ERR_ARG, "depth of field needs a nonzero focus_z");
    const fvc_int2 res = info->cam_info.resolution;
    if (res.x <= 0 || res.y <= 0 || (long long)res.x * res.y > (1ll << 30)) return fail(FVC_ERR_ARG, "bad resolution");
    return FVC_OK;
}

/* The head input layout each variant produces must match the model's
 * latent_offset: DensityIntermediates puts the density in latent 0 (a model
 * whose first latent is the density), the others put log-density in row 0
 * ahead of the latents (a model whose first latent is not).  eval picks the
 * variant from the model the same way (src/eval.cu:215-222). */
static int check_variant(const fvc_renderer *r)
{
    /* the cache stores 8 latents per voxel (two half4 arrays, include/cache.h:24-27) */
    if (r->m->n_latents > 8)
        return fail(FVC_ERR_CONFIG, "the cache stores 8 latents per voxel; this model's head reads " +
                                        std::to_string(r->m->n_latents));
    /* the basic cache renderer puts its 8 interpolated intermediates where the
     * head reads them whatever the variant (src/cache_basic_renderer.cu:187) */
    if (r->kind == FVC_RENDERER_CACHE_BASIC) return FVC_OK;
    const bool di = r->settings.interpol_variant == VARIANT_DENSITY_INTERMEDIATES;
    if (di && r->m->latent_offset != 0)
        return fail(FVC_ERR_CONFIG, "the DensityIntermediates cache variant needs a model whose first latent is the density");
    if (!di && r->m->latent_offset != 1)
        return fail(FVC_ERR_CONFIG, "the " + std::string(r->settings.interpol_variant == VARIANT_DENSITY ? "Density" : "Alpha") +
                                        " cache variants need a model whose first latent is not the density "
                                        "(use DensityIntermediates)");
    return FVC_OK;
}

static void apply_settings(const fvc_renderer *r, CacheView &v)
{
    const fvc_cache_settings &c = r->settings;
    v.interp = c.interpol_function;
    v.first_latent_is_density = c.interpol_variant == VARIANT_DENSITY_INTERMEDIATES;
    v.variant = c.interpol_variant;
    v.reweight = c.reweight_intermediates ? 1 : 0;
    v.keep_first = c.disable_reweighting_first_intermediate ? 1 : 0;
    v.inter_brick = c.use_inter_brick_interpolation ? 1 : 0;
}

static int setup_render_params(fvc_renderer *r, const fvc_raymarch_info *info, float4 *results, uchar4 *image, int4 *counts,
                               RenderParams &p, bool per_view_caches = false)
{
    fvc_model *m = r->m;
    const bool cached = is_cache_kind(r->kind);
    memset(&p, 0, sizeof(p));
    p.scene = m->dscene;
    p.steps = dev_steps(info->stepsize_info);
    p.cam = dev_cam_rm(*info);
    p.grid = m->grid;
    p.bits = m->d_bits; p.table = m->d_table; p.weights = m->d_weights; p.bias3 = m->d_bias3;
    p.weights_tc = m->d_weights_tc;
    p.use_tc = r->use_tc;
    p.precision = r->precision;
    p.weights_tc_bf16 = m->d_weights_tc_bf16;
    p.weights_tc_fp8 = m->d_weights_tc_fp8;
    p.tc_fp8_iw = m->d_fp8_iw;
    if (r->precision != FVC_PRECISION_FP16 && (cached || !r->use_tc))
        return fail(FVC_ERR_CONFIG, "BF16 and FP8 MLPs are built for the plain renderers on the tcgen05 network path");
    if (m->view_dependent && (!r->use_tc || r->precision != FVC_PRECISION_FP16))
        return fail(FVC_ERR_CONFIG, "view-dependent models (mlp_first_head) are built for the renderers and cache builds on the tcgen05 network path in FP16 (the autotuner also tries the mma.sync path)");
    p.view_dependent = m->view_dependent;
    p.weights_vd = m->d_weights_vd;
    p.latent_offset = m->latent_offset;
    if (m->freq && (!r->use_tc || r->precision != FVC_PRECISION_FP16 || r->m_tile != 128))
        return fail(FVC_ERR_CONFIG, "heads with the frequency encoding are built for the tcgen05 network path in FP16 on 128-row tiles");
    set_head_layout(*m, p);
    p.basic_cache = r->kind == FVC_RENDERER_CACHE_BASIC;
    p.ray_counter = r->d_ctl; p.guard = r->d_ctl + 1; p.stats = r->d_stats;
    p.results = results; p.image = image; p.ray_counts = counts;
    p.sample_index = info->sample_index;
    p.max_rounds = 1 << 26;
    p.max_samples_per_ray = r->max_samples;
    if (cached) {
        int rc;
        if ((rc = check_variant(r))) return rc;
        p.render_mode = r->render_mode;
        if (!per_view_caches) {
            fvc_cache *c = r->cache;
            if (!c || !c->initialized || !c->built) return fail(FVC_ERR_CACHE_UNINIT, "Cache is not initialized!");
            p.ccam = dev_cam(c->rm_info.cam_info);
            p.csteps = dev_steps(c->rm_info.stepsize_info);
            p.cache = c->view();
            apply_settings(r, p.cache);
        }
    }
    if (info->cam_info.resolution.x != r->W || info->cam_info.resolution.y != r->H) {
        const int rc = fvc_renderer_resize(r, info->cam_info.resolution.x, info->cam_info.resolution.y);
        if (rc) return rc;
    }
    p.states[0] = r->d_states[0]; p.states[1] = r->d_states[1];
    p.ray_rows = r->d_ray_rows;
    p.row_t0 = r->d_row_t0; p.row_slot = r->d_row_slot; p.row_kind = r->d_row_kind;
    p.row_pay = r->d_row_pay; p.row_out = r->d_row_out; p.row_lat = r->d_row_lat;
    p.res_list = r->d_res_list; p.cache_list = r->d_cache_list;
    p.counters = r->d_wf_counters;
    p.row_capacity = r->row_capacity;
    p.steps_per_iter = r->steps_per_iter;
    p.m_tile = r->m_tile;
    p.fused_classify = r->fused_classify;
    p.skip_empty = r->skip_empty;
    p.row_target = std::min(r->row_target, r->row_capacity);
    return FVC_OK;
}

static void reset_launch_log(fvc_renderer *r)
{
    r->log.launches = 0;
    r->log.n_timed = r->log.n_untimed = 0;
    r->log.split = -1;
    r->log.ev = r->events.empty() ? nullptr : r->events.data();
    r->log.cap = (int)r->events.size() / 2;
}

static int enqueue_render(fvc_renderer *r, const fvc_raymarch_info *info, float4 *results, uchar4 *image, int4 *counts,
                          float *contrib_res = nullptr, float *contrib_cache = nullptr)
{
    fvc_model *m = r->m;
    const bool cached = is_cache_kind(r->kind);
    RenderParams p;
    int rc;
    if ((rc = setup_render_params(r, info, results, image, counts, p))) return rc;
    p.contrib_res = contrib_res;
    p.contrib_cache = contrib_cache;
    CU(cudaMemsetAsync(r->d_ctl, 0, 4 * sizeof(int), r->stream));
    CU(cudaMemsetAsync(r->d_stats, 0, sizeof(RenderStatsDev), r->stream));
    CU(cudaMemsetAsync(r->d_wf_counters, 0, 8 * sizeof(int), r->stream));
    reset_launch_log(r);
    r->last_was_graph = false;
    CU(render_frame(p, cached, m->head_hidden, m->n_sms, r->stream, r->h_pinned + 8, 4, &r->last_iterations, &r->log));
    return FVC_OK;
}

extern "C" int fvc_render_device(fvc_renderer *r, const fvc_raymarch_info *info, const fvc_render_outputs *out)
{
    CHECK_ARG(r && info, "fvc_render_device: null argument");
    CHECK_ARG(!out || (!out->contrib_resample && !out->contrib_cache) || is_cache_kind(r->kind),
              "fvc_render_device: contribution buffers are written by the cache renderers");
    int rc;
    if ((rc = check_info(info))) return rc;
    std::lock_guard<std::mutex> lk(r->read_mutex);
    return enqueue_render(r, info, out ? (float4 *)out->results : nullptr, out ? (uchar4 *)out->image_rgba8 : nullptr,
                          out ? (int4 *)out->ray_counts : nullptr, out ? out->contrib_resample : nullptr,
                          out ? out->contrib_cache : nullptr);
}

extern "C" int fvc_render(fvc_renderer *r, const fvc_raymarch_info *info, const fvc_render_outputs *out)
{
    CHECK_ARG(r && info, "fvc_render: null argument");
    CHECK_ARG(!out || (!out->contrib_resample && !out->contrib_cache),
              "fvc_render: contribution buffers are device buffers (fvc_render_device)");
    int rc;
    if ((rc = check_info(info))) return rc;
    if ((rc = fvc_renderer_resize(r, info->cam_info.resolution.x, info->cam_info.resolution.y))) return rc;
    std::lock_guard<std::mutex> lk(r->read_mutex);
    const size_t n = (size_t)r->W * r->H;
    if (out && out->image_rgba8 && info->sample_index > 0)
        CU(cudaMemcpyAsync(r->d_image, out->image_rgba8, n * 4, cudaMemcpyHostToDevice, r->stream));
    if ((rc = enqueue_render(r, info, r->d_results, r->d_image, r->d_counts))) return rc;
    if (out && out->results) CU(cudaMemcpyAsync(out->results, r->d_results, n * 16, cudaMemcpyDeviceToHost, r->stream));
    if (out && out->image_rgba8) CU(cudaMemcpyAsync(out->image_rgba8, r->d_image, n * 4, cudaMemcpyDeviceToHost, r->stream));
    if (out && out->ray_counts) CU(cudaMemcpyAsync(out->ray_counts, r->d_counts, n * 16, cudaMemcpyDeviceToHost, r->stream));
    CU(cudaStreamSynchronize(r->stream));
    return FVC_OK;
}

extern "C" int fvc_render_stats(fvc_renderer *r, fvc_render_stats_t *o)
{
    CHECK_ARG(r && o, "fvc_render_stats: null argument");
    RenderStatsDev s;
    int ctl[4];
    CU(cudaStreamSynchronize(r->stream));
    CU(cudaMemcpy(&s, r->d_stats, sizeof(s), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(ctl, r->d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost));
    const double n_rays = (double)std::max(1, r->W * r->H);
    o->n_samples = (long long)s.n_samples;
    o->n_resamples = (long long)s.n_resamples;
    o->n_cache_hits = (long long)s.n_cache_hits;
    o->n_dropped = (long long)s.n_dropped;
    o->n_steps = (long long)s.n_steps;
    o->n_rounds = r->last_iterations;
    o->samples_ppx = (double)s.n_samples / n_rays;
    o->guard_flags = ctl[1];
    o->n_launches = r->log.launches;
    if (r->last_was_graph) { /* the device loop: prologue + one body per two sub-iterations */
        int iters = 0;
        CU(cudaMemcpy(&iters, r->d_wf_counters + 5, sizeof(int), cudaMemcpyDeviceToHost));
        o->n_rounds = iters;
        o->n_launches = 1 + (long long)(r->graph_kernels - 1) * (iters / 2);
    }
    o->n_miss_outside_fov = (long long)s.n_reason[REASON_OUTSIDE_FOV];
    o->n_miss_outside_depth = (long long)s.n_reason[REASON_OUTSIDE_DEPTH];
    o->n_miss_before_near = (long long)s.n_reason[REASON_BEFORE_NEAR];
    o->n_miss_beyond_known = (long long)s.n_reason[REASON_BEYOND_KNOWN];
    o->n_drop_brick_unset = (long long)s.n_reason[REASON_BRICK_UNSET];
    o->n_drop_voxel_empty = (long long)s.n_reason[REASON_VOXEL_EMPTY];
    o->n_drop_alpha = (long long)s.n_reason[REASON_ALPHA];
    const int n_timed = r->log.ev ? r->log.n_timed : 0;
    const int split = r->log.split >= 0 ? std::min(r->log.split, n_timed) : n_timed;
    o->n_timed_launches = split;
    o->n_timed_adjoint_launches = n_timed - split;
    o->timed_kernel_ms = 0.0f;
    o->timed_adjoint_ms = 0.0f;
    for (int i = 0; i < n_timed; ++i) {
        float ms = 0.0f;
        CU(cudaEventElapsedTime(&ms, r->log.ev[2 * i], r->log.ev[2 * i + 1]));
        (i < split ? o->timed_kernel_ms : o->timed_adjoint_ms) += ms;
    }
    return FVC_OK;
}

extern "C" int fvc_model_properties(const fvc_model *m, fvc_model_props *o)
{
    CHECK_ARG(m && o, "fvc_model_properties: null argument");
    o->first_latent_is_density = m->latent_offset == 0;
    o->head_hidden_layers = m->head_hidden;
    o->n_levels = m->grid.n_levels;
    o->n_latents = m->n_latents;
    o->occupancy_bitfield = m->d_bits;
    const size_t R = (size_t)m->scene.grid_resolution;
    o->occupancy_bytes = R * R * R * (size_t)m->scene.grid_nlvl / 8;
    return FVC_OK;
}

extern "C" int fvc_renderer_synchronize(fvc_renderer *r)
{
    CHECK_ARG(r, "fvc_renderer_synchronize: null renderer");
    CU(cudaStreamSynchronize(r->stream));
    int guard = 0;
    CU(cudaMemcpy(&guard, r->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (guard) return fail(FVC_ERR_GUARD, "render guard fired: flags " + std::to_string(guard));
    return FVC_OK;
}

extern "C" int fvc_renderer_set_kernel_timing(fvc_renderer *r, int enable)
{
    CHECK_ARG(r && (enable == 0 || enable == 1), "fvc_renderer_set_kernel_timing: bad arguments");
    std::lock_guard<std::mutex> lk(r->read_mutex);
    CU(cudaStreamSynchronize(r->stream));
    if (enable && r->events.empty()) {
        r->events.resize(2 * 4096);
        for (auto &e : r->events) CU(cudaEventCreate(&e));
    } else if (!enable) {
        for (cudaEvent_t e : r->events) cudaEventDestroy(e);
        r->events.clear();
    }
    r->log.ev = nullptr;
    r->log.n_timed = 0;
    return FVC_OK;
}

/* ------------------------------------------------------------------------ */
/* cache                                                                     */
/* ------------------------------------------------------------------------ */
extern "C" int fvc_cache_create(fvc_cache **out)
{
    CHECK_ARG(out, "fvc_cache_create: null argument");
    *out = new fvc_cache();
    return FVC_OK;
}

extern "C" void fvc_cache_destroy(fvc_cache *c) { delete c; }

extern "C" int fvc_renderer_set_caches(fvc_renderer *r, fvc_cache *cache, fvc_cache *next)
{
    CHECK_ARG(r && cache && next, "fvc_renderer_set_caches: null argument");
    std::scoped_lock lk(r->read_mutex, r->write_mutex);
    r->cache = cache;
    r->next = next;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_cache_settings(fvc_renderer *r, const fvc_cache_settings *s)
{
    CHECK_ARG(r && s, "fvc_renderer_set_cache_settings: null argument");
    if (s->interpol_function < INTERP_LINEAR || s->interpol_function > INTERP_NEAREST)
        return fail(FVC_ERR_ARG, "fvc_renderer_set_cache_settings: unknown InterpolFunction");
    if (s->interpol_variant < VARIANT_DENSITY || s->interpol_variant > VARIANT_ALPHA_INTERMEDIATES)
        return fail(FVC_ERR_ARG, "fvc_renderer_set_cache_settings: unknown DensityInterpolVariant");
    /* the performance renderer never writes the density slot in this variant,
     * so it classifies no sample as a cache sample */
    if (s->interpol_variant == VARIANT_INTERMEDIATES && r->kind != FVC_RENDERER_CACHE_BASIC)
        return fail(FVC_ERR_CONFIG, "the Intermediates variant stores no density, which the cached performance renderer "
                                    "needs to classify cache samples");
    /* reweight_intermediates, disable_reweighting_first_intermediate and
     * use_inter_brick_interpolation steer the basic cache renderer only; the
     * performance renderer ignores them, as the reference's does.  use_hw_interpol
     * is unused in both (the texture fetches decide, include/raymarch_common.h:
     * 420-424) */
    r->settings = *s;
    return FVC_OK;
}


/* Cache::resize (src/cache.cu:44-84) with the sizing of
 * CacheRenderer::resizeCache (src/cache_renderer.cu:832-846). */
static int cache_resize(fvc_renderer *r, fvc_cache *c, int W, int H, const fvc_stepsize_info &st)
{
    const long long n_rays = (long long)W * H;
    /* INIT_ESTIMATED_N_SAMPLES_PER_RAY (32) and INIT_ESTIMATED_BRICK_SPARSITY (0.5), include/cache.h:14-15,
     * unless fvc_cache_set_sizing changed them */
    const long long est_samples = n_rays * r->cache_est_samples;
    const int est_per_brick = (int)(r->cache_sparsity * std::pow(8.0f, 3.0f));
    const long long est_bricks = est_samples / std::max(1, est_per_brick);
    const fvc_scene_info &s = r->m->scene;
    const float dx = s.aabb_to.x - s.aabb_from.x, dy = s.aabb_to.y - s.aabb_from.y, dz = s.aabb_to.z - s.aabb_from.z;
    const float diag = sqrtf(dx * dx + dy * dy + dz * dz);       /* max_step_in_scene */
    const float tq = diag + st.near_;
    float msteps;
    if (st.cone_angle <= 0.0f) msteps = tq / st.dt_min;
    else if (tq >= st.t_max) msteps = (tq - st.t_max) / st.dt_max + st.i_max;
    else if (tq < st.t_min) msteps = tq / st.dt_min;
    else msteps = fvc_logf(tq / st.t_min) / st.log1p_c + st.i_min;
    const int max_n_steps = (int)std::ceil(msteps);
    const int depth = (max_n_steps + 3) / 4 * 4;
    const int bX = (W + 7) / 8, bY = (H + 7) / 8, bZ = (depth + 7) / 8;
    const int dX = 128, dY = 128, dZ = (int)((est_bricks + dX * dY - 1) / (dX * dY));
    if (dZ > 1024) return fail(FVC_ERR_ARG, "fvc_cache_resize: the sizing asks for more than 128 x 128 x 1024 bricks");
    if (c->initialized && c->fW == W && c->fH == H && c->fD == depth && c->dZ == dZ) return FVC_OK;
    dfree(c->d_packed); dfree(c->d_known);
    if (c->d_voxels) cudaFree(c->d_voxels);
    c->d_voxels = nullptr;
    c->initialized = false;
    c->built = false;
    int rc;
    if ((rc = dalloc(&c->d_packed, (size_t)bX * bY * bZ, "brick index"))) return rc;
    if ((rc = dalloc(&c->d_known, (size_t)W * H, "known ranges"))) return rc;
    cudaError_t e = cudaMalloc(&c->d_voxels, (size_t)dX * dY * dZ * 512 * 32);
    if (e != cudaSuccess) { cudaGetLastError(); c->d_voxels = nullptr; return fail(FVC_ERR_OOM, "cudaMalloc cache data array"); }
    c->fW = W; c->fH = H; c->fD = depth; c->bX = bX; c->bY = bY; c->bZ = bZ; c->dX = dX; c->dY = dY; c->dZ = dZ;
    c->initialized = true;
    return FVC_OK;
}

extern "C" int fvc_cache_set_sizing(fvc_renderer *r, int est_samples_per_ray, float brick_sparsity)
{
    CHECK_ARG(r && est_samples_per_ray >= 1 && est_samples_per_ray <= 4096 && brick_sparsity > 0.0f && brick_sparsity <= 1.0f,
              "fvc_cache_set_sizing: est_samples_per_ray in [1, 4096], brick_sparsity in (0, 1]");
    r->cache_est_samples = est_samples_per_ray;
    r->cache_sparsity = brick_sparsity;
    return FVC_OK;
}

extern "C" int fvc_cache_resize(fvc_renderer *r, int width, int height, const fvc_stepsize_info *steps)
{
    CHECK_ARG(r && r->next && steps && width > 0 && height > 0, "fvc_cache_resize: bad arguments (caches attached?)");
    std::lock_guard<std::mutex> lk(r->write_mutex);
    return cache_resize(r, r->next, width, height, *steps);
}

extern "C" int fvc_cache_swap(fvc_renderer *r)
{
    CHECK_ARG(r && r->cache && r->next, "fvc_cache_swap: caches not attached");
    std::scoped_lock lk(r->read_mutex, r->write_mutex);
    std::swap(r->cache, r->next);
    return FVC_OK;
}

static int ensure_build_scratch(fvc_renderer *r, int n_tiles)
{
    BuildScratch &b = r->bs;
    if (b.n_tiles == n_tiles) return FVC_OK;
    b.release();
    int rc;
    if ((rc = dalloc(&b.rays, (size_t)n_tiles * 64, "build rays"))) return rc;
    if ((rc = dalloc(&b.block_step, (size_t)n_tiles, "block steps"))) return rc;
    if ((rc = dalloc(&b.tile_alive, (size_t)n_tiles, "tile alive"))) return rc;
    if ((rc = dalloc(&b.alive_a, (size_t)n_tiles, "alive list"))) return rc;
    if ((rc = dalloc(&b.alive_b, (size_t)n_tiles, "alive list"))) return rc;
    if ((rc = dalloc(&b.counters, (size_t)8, "build counters"))) return rc;
    if ((rc = dalloc(&b.tile_n_samples, (size_t)n_tiles, "tile samples"))) return rc;
    if ((rc = dalloc(&b.tile_processed, (size_t)n_tiles, "tile flags"))) return rc;
    if ((rc = dalloc(&b.tile_need, (size_t)n_tiles, "tile flags"))) return rc;
    if ((rc = dalloc(&b.tile_n_alive, (size_t)n_tiles, "tile alive counts"))) return rc;
    if ((rc = dalloc(&b.jobs, (size_t)2 * n_tiles, "fill jobs"))) return rc;
    if ((rc = dalloc(&b.rows, (size_t)n_tiles * 512, "build rows"))) return rc;
    if ((rc = dalloc(&b.den, (size_t)n_tiles * 512, "build densities"))) return rc;
    if ((rc = dalloc(&b.lat, (size_t)n_tiles * 512, "build latents"))) return rc;
    if ((rc = dalloc(&b.row_of, (size_t)n_tiles * 512, "build row map"))) return rc;
    b.n_tiles = n_tiles;
    return FVC_OK;
}

/* CacheRenderer::initCacheBlockwise, src/cache_renderer.cu:931-1051 */
extern "C" int fvc_cache_build(fvc_renderer *r, const fvc_raymarch_info *info)
{
    CHECK_ARG(r && info, "fvc_cache_build: null argument");
    CHECK_ARG(r->next, "fvc_cache_build: caches not attached (fvc_renderer_set_caches)");
    int rc;
    if ((rc = check_info(info, true))) return rc;
    fvc_model *m = r->m;
    if ((rc = check_variant(r))) return rc;
    std::lock_guard<std::mutex> lk(r->write_mutex);
    fvc_cache *c = r->next;
    const int W = info->cam_info.resolution.x, H = info->cam_info.resolution.y;
    if ((rc = cache_resize(r, c, W, H, info->stepsize_info))) return rc;
    c->rm_info = *info;
    c->built = false;
    const int n_tiles = c->bX * c->bY;
    if ((rc = ensure_build_scratch(r, n_tiles))) return rc;
    BuildScratch &b = r->bs;
    /* the build runs on the renderer's lowest-priority stream, as the
     * reference's _low_priority_stream (src/cache_renderer.cu:937-1044), so a
     * build called from another thread overlaps the renders on `stream`.  It
     * first waits for the work already queued there, which may still read the
     * cache being rebuilt; it returns once the build has finished. */
    cudaStream_t s = r->low_prio;
    CU(cudaEventRecord(r->build_after, r->stream));
    CU(cudaStreamWaitEvent(s, r->build_after, 0));

    CacheBuildParams p;
    memset(&p, 0, sizeof(p));
    p.scene = m->dscene; p.steps = dev_steps(info->stepsize_info); p.cam = dev_cam(info->cam_info); p.grid = m->grid;
    p.bits = m->d_bits; p.table = m->d_table; p.weights = m->d_weights; p.latent_offset = m->latent_offset;
    p.variant = r->settings.interpol_variant;
    p.view_dependent = m->view_dependent;
    p.weights_fh = m->d_weights_fh;
    if (m->view_dependent) {
        if (!b.dirs && (rc = dalloc(&b.dirs, (size_t)n_tiles * 512, "build ray directions"))) return rc;
        p.build_dirs = b.dirs;
    }
    p.bX = c->bX; p.bY = c->bY; p.bZ = c->bZ; p.fW = c->fW; p.fH = c->fH; p.fD = c->fD;
    p.dX = c->dX; p.dY = c->dY; p.dZ = c->dZ; p.capacity = c->capacity();
    p.rays = b.rays; p.block_step = b.block_step; p.tile_alive = b.tile_alive;
    p.alive_list = b.alive_a; p.alive_list_next = b.alive_b;
    p.n_alive_tiles = b.counters + 0; p.n_alive_next = b.counters + 1;
    p.slot_counter = b.counters + 2; p.n_jobs = b.counters + 3; p.guard = b.counters + 4;
    p.tile_n_samples = b.tile_n_samples; p.tile_processed = b.tile_processed; p.tile_need = b.tile_need;
    p.tile_n_alive = b.tile_n_alive; p.voxels = c->d_voxels;
    p.packed_index = c->d_packed; p.known_ranges = c->d_known; p.jobs = b.jobs;
    p.max_search = c->bZ + 4;
    p.build_rows = b.rows; p.build_den = b.den; p.build_lat = b.lat; p.build_row_of = b.row_of;
    p.build_row_counter = b.counters + 5;

    CU(cudaMemsetAsync(b.counters, 0, 8 * sizeof(int), s));
    CU(cudaMemsetAsync(c->d_packed, 0xff, (size_t)c->bX * c->bY * c->bZ * sizeof(int32_t), s));
    int n_launches = 2;
    cache_init_kernel<<<n_tiles, 64, 0, s>>>(p);
    CU(cudaGetLastError());
    cache_compact_kernel<<<1, 1024, 0, s>>>(p, n_tiles);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(r->h_pinned, b.counters, sizeof(int), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    int n_alive = r->h_pinned[0];
    long long n_samples = 0;
    int iter = 0;
    const int max_iter = c->bZ + 8;
    std::vector<int> dummy;
    for (; iter < max_iter && n_alive > 0; ++iter) {
        CU(cudaMemsetAsync(p.build_row_counter, 0, sizeof(int), s));
        CU(launch_cache_search(p, std::min(n_alive, 1 << 16), s));
        CU(cudaGetLastError());
        /* the density network (fvc_renderer_set_build_network_path); view-dependent models' first head runs
         * in the warp-level kernel */
        if (r->build_tc && !m->view_dependent) CU(launch_cache_density_tc(p, m->d_weights_tc, m->n_sms, s));
        else CU(launch_cache_density(p, m->n_sms * 8, s));
        CU(cudaGetLastError());
        cache_composite_kernel<<<std::min((n_alive + 3) / 4, 1 << 16), 128, 0, s>>>(p);
        CU(cudaGetLastError());
        cache_assign_kernel<<<1, 1024, 0, s>>>(p);
        CU(cudaGetLastError());
        cache_fill_kernel<<<std::min(n_alive, 8 * m->n_sms), 256, 0, s>>>(p);
        CU(cudaGetLastError());
        n_launches += 5;
        std::swap(p.alive_list, p.alive_list_next);
        std::swap(p.n_alive_tiles, p.n_alive_next);
        CU(cudaMemcpyAsync(r->h_pinned, p.n_alive_tiles, sizeof(int), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        n_alive = r->h_pinned[0];
    }
    cache_known_ranges_kernel<<<n_tiles, 64, 0, s>>>(p);
    CU(cudaGetLastError());
    ++n_launches;
    CU(cudaMemcpyAsync(r->h_pinned, b.counters, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    const int demanded = r->h_pinned[2], guard = r->h_pinned[4];
    c->stats.n_bricks_demanded = demanded;
    c->stats.n_bricks_reserved = c->capacity();
    c->stats.n_bricks_set = std::min(demanded, c->capacity());
    c->stats.overflow = demanded > c->capacity();
    c->stats.n_iterations = iter;
    c->stats.n_launches = n_launches;
    c->stats.n_samples = n_samples;
    c->built = true;
    if (guard) return fail(FVC_ERR_GUARD, "cache build guard fired: flags " + std::to_string(guard));
    if (n_alive > 0) return fail(FVC_ERR_GUARD, "cache build did not converge within the frustum depth");
    return FVC_OK;
}

/* CacheRenderer::initCache, src/cache_renderer.cu:848-928: the per-ray fill
 * of the "next" cache.  The cache camera's rays march like a plain render,
 * TARGET_BATCH_SIZE / alive (1..8) occupied samples per ray and sub-iteration;
 * each sub-iteration marks the bricks of the visible samples, reserves slots
 * for the new ones and writes the voxels (see PerRayFillParams).  Slots are
 * reserved per sub-iteration in (brick column, depth) order instead of by
 * atomicAdd, so the fill is reproducible. */
extern "C" int fvc_cache_build_per_ray(fvc_renderer *r, const fvc_raymarch_info *info)
{
    CHECK_ARG(r && info, "fvc_cache_build_per_ray: null argument");
    CHECK_ARG(r->next, "fvc_cache_build_per_ray: caches not attached (fvc_renderer_set_caches)");
    int rc;
    if ((rc = check_info(info, true))) return rc;
    fvc_model *m = r->m;
    if ((rc = check_variant(r))) return rc;
    std::scoped_lock lk(r->read_mutex, r->write_mutex); /* the fill runs on the renderer's wavefront buffers */
    fvc_cache *c = r->next;
    const int W = info->cam_info.resolution.x, H = info->cam_info.resolution.y;
    if ((rc = cache_resize(r, c, W, H, info->stepsize_info))) return rc;
    c->rm_info = *info;
    c->built = false;
    RenderParams p;
    if ((rc = setup_render_params(r, info, nullptr, nullptr, nullptr, p, true))) return rc;
    p.steps_per_iter = 1 << 30; /* sample_common_kernel marches until it has its samples */
    PerRayScratch &x = r->pr;
    const size_t n_bricks = (size_t)c->bX * c->bY * c->bZ, n_cols = (size_t)c->bX * c->bY, n_rows = (size_t)r->row_capacity;
    if (x.n_bricks < n_bricks || x.n_cols < n_cols || x.n_rows < n_rows) {
        x.release();
        if ((rc = dalloc(&x.flag, n_bricks, "fill brick marks"))) return rc;
        if ((rc = dalloc(&x.set, n_bricks, "fill brick flags"))) return rc;
        if ((rc = dalloc(&x.col_count, n_cols, "fill column counts"))) return rc;
        if ((rc = dalloc(&x.col_base, n_cols, "fill column bases"))) return rc;
        if ((rc = dalloc(&x.slots, (size_t)2, "fill slot counter"))) return rc;
        if ((rc = dalloc(&x.den, n_rows, "fill densities"))) return rc;
        if ((rc = dalloc(&x.lat, n_rows, "fill latents"))) return rc;
        x.n_bricks = n_bricks; x.n_cols = n_cols; x.n_rows = n_rows;
    }
    PerRayFillParams f;
    memset(&f, 0, sizeof(f));
    f.scene = m->dscene; f.steps = p.steps; f.W = W; f.H = H;
    f.states[0] = p.states[0]; f.states[1] = p.states[1];
    f.ray_rows = p.ray_rows; f.row_t0 = p.row_t0; f.den = x.den; f.lat = x.lat; f.counters = p.counters;
    f.flag = x.flag; f.set = x.set; f.packed_index = c->d_packed; f.known_ranges = c->d_known; f.voxels = c->d_voxels;
    f.bX = c->bX; f.bY = c->bY; f.bZ = c->bZ; f.dX = c->dX; f.dY = c->dY; f.dZ = c->dZ; f.capacity = c->capacity();
    f.variant = r->settings.interpol_variant;
    f.slot_counter = x.slots; f.col_count = x.col_count; f.col_base = x.col_base;
    CacheBuildParams q; /* the density network over the sub-iteration's rows */
    memset(&q, 0, sizeof(q));
    q.grid = m->grid; q.table = m->d_table; q.weights = m->d_weights; q.latent_offset = m->latent_offset;
    q.build_rows = p.row_pay; q.build_den = x.den; q.build_lat = x.lat; q.build_row_counter = p.counters + 2;
    q.view_dependent = m->view_dependent; q.weights_fh = m->d_weights_fh; q.dir_slot = p.row_slot; q.guard = p.guard;
    cudaStream_t s = r->stream;
    CU(cudaMemsetAsync(x.flag, 0, n_bricks, s));
    CU(cudaMemsetAsync(x.set, 0, n_bricks, s));
    CU(cudaMemsetAsync(x.slots, 0, 2 * sizeof(int), s));
    CU(cudaMemsetAsync(c->d_packed, 0xff, n_bricks * sizeof(int32_t), s));
    CU(cudaMemsetAsync(r->d_ctl, 0, 4 * sizeof(int), s));
    CU(cudaMemsetAsync(r->d_stats, 0, sizeof(RenderStatsDev), s));
    CU(cudaMemsetAsync(p.counters, 0, 8 * sizeof(int), s));
    const int n_sms = m->n_sms;
    pr_known_init_kernel<<<n_sms * 4, 256, 0, s>>>(f);
    CU(launch_fill_raygen(p, s));
    int n_launches = 2;
    CU(cudaMemcpyAsync(r->h_pinned, p.counters, sizeof(int), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    int n_alive = r->h_pinned[0];
    long long n_samples = 0;
    int it = 0;
    for (; it < 1000 && n_alive > 0; ++it) { /* MAX_SUBITER */
        const int n_steps = std::min(8, std::max(1, (1 << 21) / n_alive)); /* TARGET_BATCH_SIZE / n_alive */
        p.row_capacity = n_steps * n_alive;                                 /* the march gives every ray n_steps rows */
        n_samples += ((long long)n_alive * n_steps + 255) / 256 * 256;     /* next_multiple(batch, 256) */
        CU(cudaMemsetAsync(p.counters + 2, 0, sizeof(int), s));
        CU(launch_fill_march(p, it, n_sms, s));
        q.dir_states = p.states[it & 1];
        if (r->build_tc && !m->view_dependent) CU(launch_cache_density_tc(q, m->d_weights_tc, n_sms, s));
        else CU(launch_cache_density(q, n_sms * 8, s));
        pr_mark_kernel<<<n_sms * 16, 128, 0, s>>>(f, it);
        pr_count_kernel<<<(int)((n_cols + 255) / 256), 256, 0, s>>>(f);
        pr_scan_kernel<<<1, 1024, 0, s>>>(f);
        pr_reserve_kernel<<<(int)((n_cols + 255) / 256), 256, 0, s>>>(f);
        pr_zero_kernel<<<n_sms * 4, 256, 0, s>>>(f);
        pr_write_kernel<<<n_sms * 16, 128, 0, s>>>(f, it);
        CU(cudaGetLastError());
        n_launches += 8;
        CU(cudaMemcpyAsync(r->h_pinned, p.counters + ((it + 1) & 1), sizeof(int), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        n_alive = r->h_pinned[0];
    }
    CU(cudaMemcpyAsync(r->h_pinned, x.slots, sizeof(int), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(r->h_pinned + 1, r->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    const int demanded = r->h_pinned[0], guard = r->h_pinned[1];
    c->stats.n_bricks_demanded = demanded;
    c->stats.n_bricks_reserved = c->capacity();
    c->stats.n_bricks_set = std::min(demanded, c->capacity());
    c->stats.overflow = demanded > c->capacity();
    c->stats.n_iterations = it;
    c->stats.n_launches = n_launches;
    c->stats.n_samples = n_samples;
    c->built = true;
    if (guard) return fail(FVC_ERR_GUARD, "per-ray cache fill guard fired: flags " + std::to_string(guard));
    return FVC_OK;
}

extern "C" int fvc_cache_stats(fvc_renderer *r, fvc_cache_stats_t *o)
{
    CHECK_ARG(r && o && r->next, "fvc_cache_stats: bad arguments");
    *o = r->next->built ? r->next->stats : (r->cache ? r->cache->stats : r->next->stats);
    return FVC_OK;
}

extern "C" int fvc_cache_dims(fvc_cache *c, fvc_int3 *fd, fvc_int3 *bd, fvc_int3 *dd)
{
    CHECK_ARG(c, "fvc_cache_dims: null cache");
    if (!c->initialized) return fail(FVC_ERR_CACHE_UNINIT, "Cache is not initialized!");
    if (fd) *fd = {c->fW, c->fH, c->fD};
    if (bd) *bd = {c->bX, c->bY, c->bZ};
    if (dd) *dd = {c->dX, c->dY, c->dZ};
    return FVC_OK;
}

extern "C" int fvc_cache_read(fvc_cache *c, int32_t *packed, size_t *packed_n, float *known, size_t *known_n, uint32_t *vox,
                              size_t *vox_n)
{
    CHECK_ARG(c, "fvc_cache_read: null cache");
    if (!c->initialized) return fail(FVC_ERR_CACHE_UNINIT, "Cache is not initialized!");
    const size_t nb = (size_t)c->bX * c->bY * c->bZ, nk = (size_t)c->fW * c->fH, nv = (size_t)c->capacity() * 512 * 8;
    if (packed_n) *packed_n = nb;
    if (known_n) *known_n = nk;
    if (vox_n) *vox_n = nv;
    CU(cudaDeviceSynchronize());
    if (packed) CU(cudaMemcpy(packed, c->d_packed, nb * 4, cudaMemcpyDeviceToHost));
    if (known) CU(cudaMemcpy(known, c->d_known, nk * 4, cudaMemcpyDeviceToHost));
    if (vox) CU(cudaMemcpy(vox, c->d_voxels, nv * 4, cudaMemcpyDeviceToHost));
    return FVC_OK;
}

/* ------------------------------------------------------------------------ */
/* views for the allocation-free render (fvc_noalloc.cu)                     */
/* ------------------------------------------------------------------------ */
namespace fvc_internal {
int model_views(const fvc_model *m, RenderParams *p, int *head_hidden, int *n_sms)
{
    if (m->view_dependent) return fail(FVC_ERR_CONFIG, "view-dependent models (mlp_first_head) are built for the renderers and cache builds on the tcgen05 network path in FP16 (the autotuner also tries the mma.sync path)");
    set_head_layout(*m, *p);
    p->scene = m->dscene;
    p->grid = m->grid;
    p->bits = m->d_bits;
    p->table = m->d_table;
    p->weights = m->d_weights;
    p->weights_tc = m->d_weights_tc;
    p->use_tc = 1;
    p->bias3 = m->d_bias3;
    p->latent_offset = m->latent_offset;
    *head_hidden = m->head_hidden;
    *n_sms = m->n_sms;
    return FVC_OK;
}
void set_error(const char *msg) { g_err = msg; }
/* the device forms of the step and camera structs, built exactly as the
 * allocating renderers build them */
DevSteps steps_view(const fvc_stepsize_info &s) { return dev_steps(s); }
DevCam cam_view(const fvc_raymarch_info &rm) { return dev_cam_rm(rm); }
}  // namespace fvc_internal

extern "C" int fvc_renderer_set_network_path(fvc_renderer *r, int use_tcgen05)
{
    CHECK_ARG(r && (use_tcgen05 == 0 || use_tcgen05 == 1), "fvc_renderer_set_network_path: bad arguments");
    r->use_tc = use_tcgen05;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_build_network_path(fvc_renderer *r, int use_tcgen05)
{
    CHECK_ARG(r && (use_tcgen05 == 0 || use_tcgen05 == 1), "fvc_renderer_set_build_network_path: bad arguments");
    r->build_tc = use_tcgen05;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_empty_space_skipping(fvc_renderer *r, int on)
{
    CHECK_ARG(r && (on == 0 || on == 1), "fvc_renderer_set_empty_space_skipping: bad arguments");
    r->skip_empty = on;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_fused_classify(fvc_renderer *r, int on)
{
    CHECK_ARG(r && (on == 0 || on == 1), "fvc_renderer_set_fused_classify: bad arguments");
    r->fused_classify = on;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_tiling(fvc_renderer *r, int m_tile, int batch_rows)
{
    CHECK_ARG(r && (m_tile == 64 || m_tile == 128 || m_tile == 256) && (batch_rows == 0 || (batch_rows >= 1024 && batch_rows <= (1 << 26))),
              "fvc_renderer_set_tiling: m_tile must be 64, 128 or 256 and batch_rows 0 or in [2^10, 2^26]");
    r->m_tile = m_tile;
    r->row_target = batch_rows;
    return FVC_OK;
}

/* ------------------------------------------------------------------------ */
/* differentiable render                                                     */
/* ------------------------------------------------------------------------ */
struct fvc_grad {
    fvc_model *m = nullptr;
    size_t n_table = 0, n_base = 0, n_head = 0;
    float *d_table = nullptr, *d_base = nullptr, *d_head = nullptr; /* dL/dparam, accumulated */
    float *s_table = nullptr, *s_base = nullptr, *s_head = nullptr; /* loss-scaled, one call */
    uint2 *d_w = nullptr;                                           /* BW_TOTAL weight packs, fp16 */
    uint2 *d_w_bf16 = nullptr;                                      /* the same in bf16 */
    uint8_t *d_wtc = nullptr, *d_wtc_bf16 = nullptr;                /* TB_BYTES K-major tiles, fp16 / bf16 */
    float4 *d_ray_grad = nullptr;
    int ray_cap = 0;
    double *d_loss = nullptr;
    float *d_lat = nullptr, *s_lat = nullptr;                       /* cache-latent gradients [slots][512][8] */
    size_t n_lat = 0;
    ~fvc_grad()
    {
        dfree(d_table); dfree(d_base); dfree(d_head); dfree(s_table); dfree(s_base); dfree(s_head);
        dfree(d_lat); dfree(s_lat);
        dfree(d_w); dfree(d_w_bf16); dfree(d_wtc); dfree(d_wtc_bf16); dfree(d_ray_grad); dfree(d_loss);
    }
};

static constexpr float FVC_LOSS_SCALE = 1024.0f;

extern "C" int fvc_grad_create(fvc_model *m, fvc_grad **out)
{
    CHECK_ARG(m && out, "fvc_grad_create: null argument");
    *out = nullptr;
    if (m->view_dependent) return fail(FVC_ERR_CONFIG, "the adjoint is built for networks without the view-dependent split head");
    if (m->freq) return fail(FVC_ERR_CONFIG, "the adjoint is built for heads without the frequency encoding");
    if (m->n_latents != 8 || m->grid.n_levels != 16)
        return fail(FVC_ERR_CONFIG, "the backward kernels are built for 16 hash levels of 2 features and 8 latents");
    auto g = std::make_unique<fvc_grad>();
    g->m = m;
    g->n_table = m->table_entries * 2;
    g->n_base = m->h_base.size();
    g->n_head = m->h_head.size();
    int rc;
    if ((rc = dalloc(&g->d_table, g->n_table, "table gradient"))) return rc;
    if ((rc = dalloc(&g->s_table, g->n_table, "table gradient"))) return rc;
    if ((rc = dalloc(&g->d_base, g->n_base, "base gradient"))) return rc;
    if ((rc = dalloc(&g->s_base, g->n_base, "base gradient"))) return rc;
    if ((rc = dalloc(&g->d_head, g->n_head, "head gradient"))) return rc;
    if ((rc = dalloc(&g->s_head, g->n_head, "head gradient"))) return rc;
    if ((rc = dalloc(&g->d_loss, (size_t)1, "loss"))) return rc;
    CU(cudaMemset(g->d_table, 0, g->n_table * 4)); CU(cudaMemset(g->s_table, 0, g->n_table * 4));
    CU(cudaMemset(g->d_base, 0, g->n_base * 4)); CU(cudaMemset(g->s_base, 0, g->n_base * 4));
    CU(cudaMemset(g->d_head, 0, g->n_head * 4)); CU(cudaMemset(g->s_head, 0, g->n_head * 4));
    /* forward (B = W^T) and input-gradient (B = W) fragment packs of each layer */
    auto slice = [](const std::vector<uint16_t> &v, size_t off, size_t n) {
        return std::vector<uint16_t>(v.begin() + off, v.begin() + off + n);
    };
    auto transpose = [](const std::vector<uint16_t> &W, int R, int Cc) {
        std::vector<uint16_t> T((size_t)R * Cc);
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < Cc; ++j) T[(size_t)j * R + i] = W[(size_t)i * Cc + j];
        return T;
    };
    auto bf16_bits = [](const std::vector<uint16_t> &v) { /* fp16 bits -> bf16 bits (round to nearest even) */
        std::vector<uint16_t> o(v.size());
        for (size_t i = 0; i < v.size(); ++i) {
            const __nv_bfloat16 b = __float2bfloat16_rn(h2f(v[i]));
            memcpy(&o[i], &b, 2);
        }
        return o;
    };
    for (int variant = 0; variant < 2; ++variant) {
        auto cv = [&](const std::vector<uint16_t> &v) { return variant ? bf16_bits(v) : v; };
        const std::vector<uint16_t> W1 = cv(slice(m->h_base, 0, 64 * 32)), W2 = cv(slice(m->h_base, 64 * 32, 16 * 64));
        const std::vector<uint16_t> W3 = cv(slice(m->h_head, 0, 64 * 32));
        const size_t w5 = m->head_hidden == 2 ? 64 * 32 + 64 * 64 : 64 * 32;
        const std::vector<uint16_t> W5 = cv(slice(m->h_head, w5, 16 * 64));
        std::vector<uint2> P(BW_TOTAL, make_uint2(0, 0));
        frag_pack(W1, 64, 32, &P[BW_F1]);
        frag_pack(W2, 16, 64, &P[BW_F2]);
        frag_pack(W3, 64, 32, &P[BW_F3]);
        frag_pack(W5, 16, 64, &P[BW_F5]);
        frag_pack(transpose(W5, 16, 64), 64, 16, &P[BW_B5]);
        frag_pack(transpose(W3, 64, 32), 32, 64, &P[BW_B3]);
        frag_pack(transpose(W2, 16, 64), 64, 16, &P[BW_B2]);
        frag_pack(transpose(W1, 64, 32), 32, 64, &P[BW_B1]);
        if (m->head_hidden == 2) {
            const std::vector<uint16_t> W4 = cv(slice(m->h_head, 64 * 32, 64 * 64));
            frag_pack(W4, 64, 64, &P[BW_F4]);
            frag_pack(transpose(W4, 64, 64), 64, 64, &P[BW_B4]);
        }
        uint2 *&dst = variant ? g->d_w_bf16 : g->d_w;
        if ((rc = dalloc(&dst, P.size(), "backward weights"))) return rc;
        CU(cudaMemcpy(dst, P.data(), P.size() * sizeof(uint2), cudaMemcpyHostToDevice));
        /* the tcgen05 kernel's weight tiles: each layer [out][in] K-major */
        std::vector<uint8_t> T(TB_BYTES, 0);
        auto put = [&](const std::vector<uint16_t> &Wm, int N, int K, int off) {
            for (int n = 0; n < N; ++n)
                for (int k = 0; k < K; ++k) memcpy(&T[off + kmajor_offset(n, k, K)], &Wm[(size_t)n * K + k], 2);
        };
        put(W1, 64, 32, TB_W1);
        put(W2, 16, 64, TB_W2);
        put(W3, 64, 32, TB_W3);
        put(W5, 16, 64, TB_W5);
        if (m->head_hidden == 2) put(cv(slice(m->h_head, 64 * 32, 64 * 64)), 64, 64, TB_W4);
        uint8_t *&dt = variant ? g->d_wtc_bf16 : g->d_wtc;
        if ((rc = dalloc(&dt, T.size(), "backward weight tiles"))) return rc;
        CU(cudaMemcpy(dt, T.data(), T.size(), cudaMemcpyHostToDevice));
    }
    *out = g.release();
    return FVC_OK;
}

extern "C" void fvc_grad_destroy(fvc_grad *g) { delete g; }

extern "C" int fvc_grad_zero(fvc_grad *g)
{
    CHECK_ARG(g, "fvc_grad_zero: null argument");
    if (g->n_lat) CU(cudaMemset(g->d_lat, 0, g->n_lat * 4));
    CU(cudaMemset(g->d_table, 0, g->n_table * 4));
    CU(cudaMemset(g->d_base, 0, g->n_base * 4));
    CU(cudaMemset(g->d_head, 0, g->n_head * 4));
    return FVC_OK;
}

extern "C" int fvc_grad_sizes(const fvc_grad *g, size_t *n_table, size_t *n_base, size_t *n_head)
{
    CHECK_ARG(g, "fvc_grad_sizes: null argument");
    if (n_table) *n_table = g->n_table;
    if (n_base) *n_base = g->n_base;
    if (n_head) *n_head = g->n_head;
    return FVC_OK;
}

extern "C" int fvc_grad_cache_latents(fvc_grad *g, float *latents, size_t *n)
{
    CHECK_ARG(g, "fvc_grad_cache_latents: null argument");
    if (n) *n = g->n_lat;
    if (latents && g->n_lat) CU(cudaMemcpy(latents, g->d_lat, g->n_lat * 4, cudaMemcpyDeviceToHost));
    return FVC_OK;
}

extern "C" int fvc_grad_read(fvc_grad *g, float *table, float *base, float *head)
{
    CHECK_ARG(g, "fvc_grad_read: null argument");
    if (table) CU(cudaMemcpy(table, g->d_table, g->n_table * 4, cudaMemcpyDeviceToHost));
    if (base) CU(cudaMemcpy(base, g->d_base, g->n_base * 4, cudaMemcpyDeviceToHost));
    if (head) CU(cudaMemcpy(head, g->d_head, g->n_head * 4, cudaMemcpyDeviceToHost));
    return FVC_OK;
}

extern "C" int fvc_render_backward(fvc_renderer *r, fvc_grad *g, const fvc_raymarch_info *info, const int32_t *pixels,
                                   int n_rays, const float *target, double *loss_out, float *pred)
{
    CHECK_ARG(r && g && info && pixels && target && n_rays > 0, "fvc_render_backward: bad arguments");
    CHECK_ARG(g->m == r->m, "fvc_render_backward: gradients belong to another model");
    const bool cached = is_cache_kind(r->kind);
    if (r->precision == FVC_PRECISION_FP8_E4M3)
        return fail(FVC_ERR_CONFIG, "fvc_render_backward: the network adjoint is built for FP16 and BF16 MLPs");
    if (r->kind == FVC_RENDERER_CACHE_BASIC)
        return fail(FVC_ERR_CONFIG, "fvc_render_backward: the cached adjoint is built for the performance cache renderer");
    int rc;
    if ((rc = check_info(info))) return rc;
    const long long n_pix = (long long)info->cam_info.resolution.x * info->cam_info.resolution.y;
    CHECK_ARG(n_rays <= n_pix, "fvc_render_backward: more rays than pixels");
    if ((rc = fvc_renderer_resize(r, info->cam_info.resolution.x, info->cam_info.resolution.y))) return rc;
    std::lock_guard<std::mutex> lk(r->read_mutex);
    fvc_model *m = r->m;
    cudaStream_t s = r->stream;
    if (r->bwd_capacity != r->row_capacity) {
        dfree(r->d_row_dout); dfree(r->d_grad_rows); dfree(r->d_grad_cache_rows);
        if ((rc = dalloc(&r->d_row_dout, (size_t)r->row_capacity, "row gradients"))) return rc;
        if ((rc = dalloc(&r->d_grad_rows, (size_t)r->row_capacity, "gradient rows"))) return rc;
        if ((rc = dalloc(&r->d_grad_cache_rows, (size_t)r->row_capacity, "gradient rows"))) return rc;
        r->bwd_capacity = r->row_capacity;
    }
    if (cached) {
        if (!r->cache || !r->cache->built) return fail(FVC_ERR_CACHE_UNINIT, "Cache is not initialized!");
        if (r->settings.interpol_variant == VARIANT_DENSITY_INTERMEDIATES)
            return fail(FVC_ERR_CONFIG, "fvc_render_backward: the cache-latent adjoint is built for the variants that keep "
                                        "the density out of the latents");
        const size_t n_lat = (size_t)r->cache->capacity() * 512 * 8;
        if (g->n_lat != n_lat) {
            dfree(g->d_lat); dfree(g->s_lat);
            g->n_lat = 0;
            if ((rc = dalloc(&g->d_lat, n_lat, "cache-latent gradient"))) return rc;
            if ((rc = dalloc(&g->s_lat, n_lat, "cache-latent gradient"))) return rc;
            CU(cudaMemset(g->d_lat, 0, n_lat * 4));
            CU(cudaMemset(g->s_lat, 0, n_lat * 4));
            g->n_lat = n_lat;
        }
    }
    if (g->ray_cap < n_rays) {
        dfree(g->d_ray_grad);
        if ((rc = dalloc(&g->d_ray_grad, (size_t)n_rays, "ray gradients"))) return rc;
        g->ray_cap = n_rays;
    }
    RenderParams p;
    if ((rc = setup_render_params(r, info, r->d_results, nullptr, nullptr, p))) return rc;
    p.pixel_list = pixels;
    p.n_list = n_rays;
    p.ray_grad = g->d_ray_grad;
    p.row_dout = r->d_row_dout;
    p.grad_res_list = r->d_grad_rows;
    p.grad_cache_list = r->d_grad_cache_rows;
    BwdParams b;
    b.w = r->precision == FVC_PRECISION_BF16 ? g->d_w_bf16 : g->d_w;
    b.wtc = r->precision == FVC_PRECISION_BF16 ? g->d_wtc_bf16 : g->d_wtc;
    b.g_table = g->s_table; b.g_base = g->s_base; b.g_head = g->s_head;
    b.head_w5 = m->head_hidden == 2 ? GH_W4 + 64 * 64 : GH_W4;
    b.loss = g->d_loss;
    b.target = target;
    b.loss_scale = FVC_LOSS_SCALE;
    b.g_lat = cached ? g->s_lat : nullptr;
    reset_launch_log(r);
    /* pass 1: forward render of the listed pixels into d_results */
    CU(cudaMemsetAsync(r->d_ctl, 0, 4 * sizeof(int), s));
    CU(cudaMemsetAsync(r->d_stats, 0, sizeof(RenderStatsDev), s));
    CU(cudaMemsetAsync(r->d_wf_counters, 0, 8 * sizeof(int), s));
    CU(render_frame(p, cached, m->head_hidden, m->n_sms, s, r->h_pinned + 8, 4, &r->last_iterations, &r->log));
    /* loss and per-ray dL/dC */
    CU(cudaMemsetAsync(g->d_loss, 0, sizeof(double), s));
    CU(launch_loss(p, b, s));
    /* pass 2: re-march, compositing adjoint, network adjoint */
    r->log.split = r->log.n_timed;
    CU(cudaMemsetAsync(r->d_wf_counters, 0, 8 * sizeof(int), s));
    CU(backward_frame(p, b, cached, m->head_hidden, m->n_sms, s, r->h_pinned + 8, 4, &r->log));
    const float inv = 1.0f / (FVC_LOSS_SCALE * (float)n_rays);
    CU(launch_grad_finalize(g->s_table, g->d_table, g->n_table, inv, m->n_sms, s));
    CU(launch_grad_finalize(g->s_base, g->d_base, g->n_base, inv, m->n_sms, s));
    CU(launch_grad_finalize(g->s_head, g->d_head, g->n_head, inv, m->n_sms, s));
    if (cached) CU(launch_grad_finalize(g->s_lat, g->d_lat, g->n_lat, inv, m->n_sms, s));
    r->log.launches += cached ? 5 : 4;
    if (pred) CU(cudaMemcpyAsync(pred, r->d_results, (size_t)n_rays * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    double loss = 0.0;
    CU(cudaMemcpyAsync(&loss, g->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    int guard = 0;
    CU(cudaMemcpy(&guard, r->d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (guard) return fail(FVC_ERR_GUARD, "render guard fired: flags " + std::to_string(guard));
    if (loss_out) *loss_out = loss / (double)n_rays;
    return FVC_OK;
}

extern "C" int fvc_renderer_set_precision(fvc_renderer *r, int precision)
{
    CHECK_ARG(r && precision >= FVC_PRECISION_FP16 && precision <= FVC_PRECISION_FP8_E4M3, "fvc_renderer_set_precision: bad arguments");
    r->precision = precision;
    return FVC_OK;
}

/* ------------------------------------------------------------------------ */
/* batched views: one graph launch per batch                                 */
/* ------------------------------------------------------------------------ */
static int batch_setup(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, const fvc_render_outputs *out,
                       RenderParams &p, int &n_rays, fvc_cache *const *caches = nullptr)
{
    CHECK_ARG(r && infos && n_views > 0, "fvc_render_batch: bad arguments");
    const bool cached = is_cache_kind(r->kind);
    if (cached != (caches != nullptr))
        return fail(FVC_ERR_CONFIG, "fvc_render_batch: plain renderers take no caches, cache renderers take one per view "
                                    "(fvc_render_batch_cached)");
    if (caches)
        for (int v = 0; v < n_views; ++v)
            if (!caches[v] || !caches[v]->initialized || !caches[v]->built)
                return fail(FVC_ERR_CACHE_UNINIT, "Cache is not initialized!");
    long long total = 0;
    int rc;
    for (int v = 0; v < n_views; ++v) {
        if ((rc = check_info(&infos[v]))) return rc;
        if (memcmp(&infos[v].stepsize_info, &infos[0].stepsize_info, sizeof(fvc_stepsize_info)) != 0)
            return fail(FVC_ERR_ARG, "fvc_render_batch: the views of a batch share one StepsizeInfo");
        total += (long long)infos[v].cam_info.resolution.x * infos[v].cam_info.resolution.y;
    }
    if (total > (1ll << 30)) return fail(FVC_ERR_ARG, "fvc_render_batch: more than 2^30 rays");
    n_rays = (int)total;
    if ((rc = fvc_renderer_resize(r, n_rays, 1))) return rc;
    if (r->views_cap < n_views) {
        dfree(r->d_views); dfree(r->d_view_off); dfree(r->d_view_caches);
        if ((rc = dalloc(&r->d_views, (size_t)n_views, "views"))) return rc;
        if ((rc = dalloc(&r->d_view_off, (size_t)n_views + 1, "view offsets"))) return rc;
        if ((rc = dalloc(&r->d_view_caches, (size_t)n_views, "view caches"))) return rc;
        r->views_cap = n_views;
    }
    if (caches) {
        std::vector<ViewCache> vcs(n_views);
        for (int v = 0; v < n_views; ++v) {
            vcs[v].cache = caches[v]->view();
            apply_settings(r, vcs[v].cache);
            vcs[v].ccam = dev_cam(caches[v]->rm_info.cam_info);
            vcs[v].csteps = dev_steps(caches[v]->rm_info.stepsize_info);
        }
        CU(cudaMemcpyAsync(r->d_view_caches, vcs.data(), vcs.size() * sizeof(ViewCache), cudaMemcpyHostToDevice, r->stream));
    }
    std::vector<DevCam> cams(n_views);
    std::vector<int> off(n_views + 1, 0);
    for (int v = 0; v < n_views; ++v) {
        cams[v] = dev_cam_rm(infos[v]);
        off[v + 1] = off[v] + infos[v].cam_info.resolution.x * infos[v].cam_info.resolution.y;
    }
    /* pageable sources: staged before the calls return, so the vectors may go */
    CU(cudaMemcpyAsync(r->d_views, cams.data(), cams.size() * sizeof(DevCam), cudaMemcpyHostToDevice, r->stream));
    CU(cudaMemcpyAsync(r->d_view_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, r->stream));
    fvc_raymarch_info first = infos[0];
    first.cam_info.resolution.x = n_rays;
    first.cam_info.resolution.y = 1;
    if ((rc = setup_render_params(r, &first, out ? (float4 *)out->results : nullptr, out ? (uchar4 *)out->image_rgba8 : nullptr,
                                  out ? (int4 *)out->ray_counts : nullptr, p, cached)))
        return rc;
    p.view_caches = caches ? r->d_view_caches : nullptr;
    p.views = r->d_views;
    p.view_off = r->d_view_off;
    p.n_views = n_views;
    p.max_iterations = 1 << 14;
    return FVC_OK;
}

static int batch_launch(fvc_renderer *r, const RenderParams &p, int n_rays)
{
    fvc_model *m = r->m;
    if (!r->graph_exec || r->graph_head_hidden != m->head_hidden || memcmp(&r->graph_params, &p, sizeof(RenderParams)) != 0) {
        if (r->graph_exec) {
            CU(cudaStreamSynchronize(r->stream));
            cudaGraphExecDestroy(r->graph_exec);
            r->graph_exec = nullptr;
        }
        CU(build_batch_graph(p, p.view_caches != nullptr, m->head_hidden, m->n_sms, r->stream, n_rays, &r->graph_exec,
                             &r->graph_kernels));
        memcpy(&r->graph_params, &p, sizeof(RenderParams));
        r->graph_head_hidden = m->head_hidden;
    }
    CU(cudaGraphLaunch(r->graph_exec, r->stream));
    reset_launch_log(r);
    r->last_was_graph = true;
    return FVC_OK;
}

extern "C" int fvc_render_batch(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, const fvc_render_outputs *out)
{
    CHECK_ARG(r, "fvc_render_batch: null renderer");
    std::lock_guard<std::mutex> lk(r->read_mutex);
    RenderParams p;
    int n_rays = 0, rc;
    if ((rc = batch_setup(r, infos, n_views, out, p, n_rays))) return rc;
    return batch_launch(r, p, n_rays);
}

extern "C" int fvc_render_batch_cached(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, fvc_cache *const *caches,
                                       const fvc_render_outputs *out)
{
    CHECK_ARG(r && caches, "fvc_render_batch_cached: null argument");
    std::lock_guard<std::mutex> lk(r->read_mutex);
    RenderParams p;
    int n_rays = 0, rc;
    if ((rc = batch_setup(r, infos, n_views, out, p, n_rays, caches))) return rc;
    return batch_launch(r, p, n_rays);
}

extern "C" int fvc_renderer_set_autotune_space(fvc_renderer *r, const int *m_tiles, int n_tiles, const int *batch_rows, int n_batches,
                                               const int *march_steps, int n_steps)
{
    CHECK_ARG(r && m_tiles && batch_rows && march_steps && n_tiles > 0 && n_tiles <= 16 && n_batches > 0 && n_batches <= 16 &&
                  n_steps > 0 && n_steps <= 16,
              "fvc_renderer_set_autotune_space: null argument or a list of 0 or more than 16 candidates");
    for (int i = 0; i < n_tiles; ++i)
        CHECK_ARG(m_tiles[i] == 32 || m_tiles[i] == 64 || m_tiles[i] == 128 || m_tiles[i] == 256,
                  "fvc_renderer_set_autotune_space: tiles must be 32 (mma.sync), 64, 128 or 256");
    for (int i = 0; i < n_batches; ++i)
        CHECK_ARG(batch_rows[i] >= 1024 && batch_rows[i] <= (1 << 26), "fvc_renderer_set_autotune_space: batches must lie in [2^10, 2^26]");
    for (int i = 0; i < n_steps; ++i)
        CHECK_ARG(march_steps[i] >= 4 && march_steps[i] <= 1024 && march_steps[i] % 4 == 0,
                  "fvc_renderer_set_autotune_space: march lengths must be multiples of 4 in [4, 1024]");
    std::lock_guard<std::mutex> lk(r->read_mutex);
    r->tune_tiles.assign(m_tiles, m_tiles + n_tiles);
    r->tune_batches.assign(batch_rows, batch_rows + n_batches);
    r->tune_steps.assign(march_steps, march_steps + n_steps);
    return FVC_OK;
}

extern "C" int fvc_renderer_autotune(fvc_renderer *r, const fvc_raymarch_info *infos, int n_views, const fvc_render_outputs *out,
                                     fvc_autotune_result *res)
{
    CHECK_ARG(r && res, "fvc_renderer_autotune: null argument");
    if (r->m->view_dependent) return fail(FVC_ERR_CONFIG, "view-dependent models (mlp_first_head) are built for the renderers and cache builds on the tcgen05 network path in FP16 (the autotuner also tries the mma.sync path)");
    if (r->m->freq) return fail(FVC_ERR_CONFIG, "heads with the frequency encoding run on 128-row tcgen05 tiles only: nothing to tune");
    std::lock_guard<std::mutex> lk(r->read_mutex);
    /* candidates: the space set by fvc_renderer_set_autotune_space (tile heights, 32 = the mma.sync warp
     * tile; compaction batches; march lengths), every combination */
    const std::vector<int> tiles = r->tune_tiles, batches = r->tune_batches, march_steps = r->tune_steps;
    const int n_ti = (int)tiles.size(), n_bi = (int)batches.size(), n_si = (int)march_steps.size();
    const int saved_tc = r->use_tc, saved_tile = r->m_tile, saved_target = r->row_target, saved_steps = r->steps_per_iter;
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_tile = 0, best_batch = 0, best_steps = 0, n_cand = 0, rc = FVC_OK;
    long long best_rows = 0;
    for (int ti = 0; ti < n_ti && rc == FVC_OK; ++ti)
        for (int bi = 0; bi < n_bi && rc == FVC_OK; ++bi)
        for (int si = 0; si < n_si && rc == FVC_OK; ++si) {
            r->use_tc = tiles[ti] != 32;
            r->m_tile = tiles[ti] == 32 ? 128 : tiles[ti];
            r->row_target = batches[bi];
            r->steps_per_iter = march_steps[si];
            RenderParams p;
            int n_rays = 0;
            if ((rc = batch_setup(r, infos, n_views, out, p, n_rays))) break;
            if ((rc = batch_launch(r, p, n_rays))) break; /* builds the graph, warms up */
            cudaEventRecord(e0, r->stream);
            for (int k = 0; k < 2 && rc == FVC_OK; ++k) rc = batch_launch(r, p, n_rays);
            cudaEventRecord(e1, r->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) { rc = fail(FVC_ERR_CUDA, "fvc_renderer_autotune: launch failed"); break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms *= 0.5f;
            ++n_cand;
            RenderStatsDev st;
            int iters = 0;
            cudaMemcpy(&st, r->d_stats, sizeof(st), cudaMemcpyDeviceToHost);
            cudaMemcpy(&iters, r->d_wf_counters + 5, sizeof(int), cudaMemcpyDeviceToHost);
            if (ms < best) {
                best = ms;
                best_tile = tiles[ti];
                best_batch = batches[bi];
                best_steps = march_steps[si];
                best_rows = (long long)st.n_samples / std::max(1, iters);
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        r->use_tc = saved_tc; r->m_tile = saved_tile; r->row_target = saved_target; r->steps_per_iter = saved_steps;
        return rc;
    }
    r->use_tc = best_tile != 32;
    r->m_tile = best_tile == 32 ? 128 : best_tile;
    r->row_target = best_batch;
    r->steps_per_iter = best_steps;
    res->m_tile = best_tile;
    res->steps_per_iter = best_steps;
    res->rows_per_iteration = best_rows;
    res->ms = best;
    res->n_candidates = n_cand;
    res->batch_rows = best_batch;
    res->reserved = 0;
    return FVC_OK;
}
