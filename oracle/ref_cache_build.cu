/*
 * ref_cache_build.cu - runs the reference's own blockwise cache-build kernels
 * on the host to make golden vectors.  TEST INFRASTRUCTURE ONLY (built by
 * oracle/Makefile into oracle/_ref/libref_cache_build.so, never part of the
 * product).
 *
 * The kernels are initPayloads_cache_init_kernel,
 * sample_cache_init_first_kernel, sample_cache_init_second_kernel,
 * accumulateNew_cache_init_second_kernel and
 * writeImageBuffer_cache_init_kernel2 (src/cache_renderer.cu:18-569).  Their
 * text is cut unchanged out of the reference file at build time (the Makefile
 * writes it into oracle/_ref/, which is not committed) and compiled here by
 * nvcc as host functions.  The reference headers (include/common.h,
 * include/raymarch_common.h, include/renderer_common.h, include/cache.h) come
 * unchanged through -I.  What a GPU would supply is emulated:
 *   - a block of 8 x 8 threads runs as 64 host threads (threadIdx / blockIdx
 *     thread-local); blocks run one after another;
 *   - __syncthreads and the cooperative-groups reduce / exclusive_scan over
 *     the 64-thread tile are barriers over those threads; __shared__
 *     variables are function statics (one block at a time);
 *   - atomicAdd is an atomic host add; surf2Dwrite / surf3Dwrite write into
 *     host arrays registered as surface handles (out-of-range writes, which
 *     a tile marching past the frustum depth makes, are counted and
 *     dropped; the golden cases keep the camera inside the scene box, where
 *     there are none);
 *   - libm stands in for the device's exp and division.
 * CacheSettings / DensityInterpolVariant come from include/cache_renderer.h,
 * which cannot be included here (it pulls in tiny-cuda-nn through
 * renderer.h); the two small definitions below repeat the reference's.
 *
 * The host loop of CacheRenderer::initCacheBlockwise
 * (src/cache_renderer.cu:931-1041: exclusive sums of the alive blocks and of
 * the per-block sample counts, the three kernels per sub-iteration, the
 * known ranges at the end) is restated by rcb_search / rcb_accumulate /
 * rcb_finish below.  The network between the search and the compositing
 * (NerfNetwork::inferenceLatents) is the caller's: rcb_search returns the
 * iteration's sample positions, the caller writes the fp16 network outputs
 * in the row-major [rows][batch] layout the kernel reads and calls
 * rcb_accumulate.
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "raymarch_common.h"
#include "renderer_common.h"
#include "cache.h"

/* include/cache_renderer.h:15-32 (see the file comment) */
enum DensityInterpolVariant
{
    Density = 0,
    Alpha = 1,
    Intermediates = 2,
    DensityIntermediates = 3,
    AlphaIntermediates = 4
};

struct CacheSettings
{
    DensityInterpolVariant interpol_variant;
    InterpolFunction interpol_function;
    bool use_hw_interpol;
    bool reweight_intermediates;
    bool disable_reweighting_first_intermediate;
    bool use_inter_brick_interpolation;
};

/* ------------------------------------------------------------------------- */
/* block emulation                                                           */
/* ------------------------------------------------------------------------- */
static constexpr int NT = Cache::PADDED_BRICK_SIZE * Cache::PADDED_BRICK_SIZE; /* threads per block */
static thread_local uint3 g_tid, g_bid;
static dim3 g_bdim;

class Barrier {
public:
    void wait()
    {
        std::unique_lock<std::mutex> lk(mu_);
        const unsigned gen = gen_;
        if (++count_ == NT) {
            count_ = 0;
            ++gen_;
            cv_.notify_all();
        } else {
            cv_.wait(lk, [&] { return gen_ != gen; });
        }
    }

private:
    std::mutex mu_;
    std::condition_variable cv_;
    int count_ = 0;
    unsigned gen_ = 0;
};
static Barrier g_barrier;
static long long g_slot[NT];

static inline int host_rank() { return (int)(g_tid.y * g_bdim.x + g_tid.x); }
static inline void host_syncthreads() { g_barrier.wait(); }

namespace hostcg {
struct thread_block {};
template <unsigned N> struct thread_block_tile {};
inline thread_block this_thread_block() { return {}; }
template <unsigned N> inline thread_block_tile<N> tiled_partition(const thread_block &) { return {}; }
template <class T> struct plus { T operator()(T a, T b) const { return a + b; } };
template <class T> struct less { T operator()(T a, T b) const { return b < a ? b : a; } };
/* reduce over the whole block (the kernels' tiles are the 64-thread block) */
template <unsigned N, class T, class Op> T reduce(const thread_block_tile<N> &, T v, Op op)
{
    static_assert(N == NT, "the cache kernels reduce over the whole 8x8 block");
    g_slot[host_rank()] = (long long)v;
    g_barrier.wait();
    T r = (T)g_slot[0];
    for (int i = 1; i < NT; ++i) r = op(r, (T)g_slot[i]);
    g_barrier.wait();
    return r;
}
template <unsigned N, class T> T exclusive_scan(const thread_block_tile<N> &, T v)
{
    static_assert(N == NT, "the cache kernels scan over the whole 8x8 block");
    const int me = host_rank();
    g_slot[me] = (long long)v;
    g_barrier.wait();
    T r = 0;
    for (int i = 0; i < me; ++i) r += (T)g_slot[i];
    g_barrier.wait();
    return r;
}
} // namespace hostcg

/* surfaces: handles into host arrays */
struct HostSurface {
    void *data = nullptr;
    size_t elem = 0;
    int dx = 0, dy = 0, dz = 0;
};
static std::vector<HostSurface> g_surf(8);
static std::atomic<long long> g_oob{0};

template <class T> static void host_surf3Dwrite(T v, cudaSurfaceObject_t s, const int3 idx)
{
    HostSurface &h = g_surf[(size_t)s];
    if (sizeof(T) != h.elem || idx.x < 0 || idx.y < 0 || idx.z < 0 || idx.x >= h.dx || idx.y >= h.dy || idx.z >= h.dz) {
        ++g_oob;
        return;
    }
    reinterpret_cast<T *>(h.data)[((size_t)idx.z * h.dy + idx.y) * h.dx + idx.x] = v;
}
template <class T> static void host_surf2Dwrite(T v, cudaSurfaceObject_t s, int x_bytes, int y)
{
    host_surf3Dwrite<T>(v, s, make_int3(x_bytes / (int)sizeof(T), y, 0));
}
static int host_atomicAdd(int *p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }

/* the reference kernels as host functions */
#undef __global__
#define __global__ static
#undef __shared__
#define __shared__ static
#define threadIdx g_tid
#define blockIdx g_bid
#define blockDim g_bdim
#define __syncthreads host_syncthreads
#define surf3Dwrite host_surf3Dwrite
#define surf2Dwrite host_surf2Dwrite
#define atomicAdd host_atomicAdd
namespace cg = hostcg;
#include "cache_build_kernels.inc"
#undef threadIdx
#undef blockIdx
#undef blockDim
#undef __syncthreads
#undef surf3Dwrite
#undef surf2Dwrite
#undef atomicAdd

/* runs fn for every thread of `n_blocks` blocks of 8 x 8 threads (block b at
 * blockIdx = (b % gx, b / gx)): 64 host threads step through the blocks
 * together, meeting at a barrier after each block so that no two blocks
 * overlap (their __shared__ statics are one block's). */
static Barrier g_block_end;
static void launch(int n_blocks, int gx, const std::function<void()> &fn)
{
    g_bdim = dim3(Cache::PADDED_BRICK_SIZE, Cache::PADDED_BRICK_SIZE, 1);
    std::vector<std::thread> ts;
    ts.reserve(NT);
    for (int k = 0; k < NT; ++k)
        ts.emplace_back([&, k] {
            g_tid = make_uint3(k % Cache::PADDED_BRICK_SIZE, k / Cache::PADDED_BRICK_SIZE, 0);
            for (int b = 0; b < n_blocks; ++b) {
                g_bid = make_uint3(b % gx, b / gx, 0);
                fn();
                g_block_end.wait();
            }
        });
    for (auto &t : ts) t.join();
}

/* ------------------------------------------------------------------------- */
/* the build (CacheRenderer::initCacheBlockwise's host loop)                  */
/* ------------------------------------------------------------------------- */
struct Build {
    RaymarchInfo rm;
    SceneInfo scene;
    CacheSettings settings;
    std::vector<uint8_t> bits;
    int3 frustum, bricks, data_bricks;
    int n_tiles, tiles_x, total_bricks, latent_offset;
    std::vector<BlockPayloadCacheInit> blocks;
    std::vector<RayPayloadCacheInit> rays;
    std::vector<int> alive, alive_idx, compact, n_steps, offsets;
    std::vector<float3> pos, dir;
    std::vector<float> t0;
    int counter = 0;
    int n_alive_blocks = 0, n_samples = 0, batch = 0;
    /* the cache's arrays (surfaces) */
    std::vector<int> packed;
    std::vector<char> isset_bricks;
    std::vector<float> isset, density, known;
    std::vector<ushort4> lat[Cache::N_DATA_ARRAYS];
    std::vector<uchar4> image;
};
static Build g;

static cudaSurfaceObject_t reg(int id, void *data, size_t elem, int dx, int dy, int dz)
{
    g_surf[id] = HostSurface{data, elem, dx, dy, dz};
    return (cudaSurfaceObject_t)id;
}

extern "C" {

/* Set-up and initPayloads_cache_init_kernel.  The reference's SceneInfo,
 * StepsizeInfo (setAdditionalInfo), CameraInfo and RaymarchInfo are built
 * from plain parameters: sc = {nlvl, contraction (0 AABB, 1 L-inf warp)},
 * f = {aabb[6], contraction aabb[6], cone, stepsize, near, far, alpha_thre,
 * fx, fy, px, py, c2w[12]}; W, H the image; bits the Morton occupancy
 * bitfield; data_bricks the data array's bricks per axis.  Returns the
 * number of 8x8 tiles, or -1. */
int rcb_init(const int *sc, const float *f, int W, int H, const uint8_t *bits, const int *data_bricks, int latent_offset, int variant)
{
    g = Build();
    const int R = 128, vals = R * R * R;
    SceneInfo si{};
    si.grid_resolution = R; si.grid_nlvl = sc[0]; si.vals_per_lvl = vals; si.normalized = false;
    si.aabb_from = make_float3(f[0], f[1], f[2]); si.aabb_to = make_float3(f[3], f[4], f[5]);
    si.contraction_aabb_from = make_float3(f[6], f[7], f[8]);
    si.contraction_aabb_to = make_float3(f[9], f[10], f[11]);
    si.contraction_type = sc[1] ? WARP_AABB_LINF : AABB;
    si.is_open_gl = false; si.alpha_thre = f[16];
    StepsizeInfo st{};
    st.cone_angle = f[12]; st.stepsize = f[13]; st.near = f[14]; st.far = f[15];
    st.setAdditionalInfo(si);
    CameraInfo ci{};
    ci.resolution = make_int2(W, H); ci.is_open_gl = false;
    ci.focal = make_float2(f[17], f[18]); ci.principal = make_float2(f[19], f[20]);
    const float *c = f + 21;
    ci.cam2world = {make_float4(c[0], c[1], c[2], c[3]), make_float4(c[4], c[5], c[6], c[7]), make_float4(c[8], c[9], c[10], c[11])};
    ci.world2cam = ci.cam2world.inverse();
    g.rm = RaymarchInfo{};
    g.rm.cam_info = ci; g.rm.next_cam_info = ci; g.rm.stepsize_info = st;
    g.rm.sample_index = 0; g.rm.motion_blur = false; g.rm.deterministic = true;
    g.scene = si;
    g.settings = CacheSettings{(DensityInterpolVariant)variant, InterpolFunction::Linear, true, true, true, true};
    g.bits.assign(bits, bits + (size_t)vals * sc[0] / 8);
    /* CacheRenderer::resizeCache (src/cache_renderer.cu:832-846) */
    const int max_n_steps = (int)ceil(max_step_in_scene(st, si));
    g.frustum = make_int3(W, H, (max_n_steps + 3) / 4 * 4);
    g.bricks = make_int3((g.frustum.x + 7) / 8, (g.frustum.y + 7) / 8, (g.frustum.z + 7) / 8);
    g.data_bricks = make_int3(data_bricks[0], data_bricks[1], data_bricks[2]);
    g.total_bricks = data_bricks[0] * data_bricks[1] * data_bricks[2];
    g.latent_offset = latent_offset;
    g.tiles_x = (W + Cache::BRICK_SIZE - 1) / Cache::BRICK_SIZE;
    const int tiles_y = (H + Cache::BRICK_SIZE - 1) / Cache::BRICK_SIZE;
    g.n_tiles = g.tiles_x * tiles_y;
    g.blocks.resize(g.n_tiles);
    g.rays.resize((size_t)g.n_tiles * NT);
    g.alive.assign(g.n_tiles, 0);
    g.alive_idx.assign(g.n_tiles, 0);
    g.compact.assign(g.n_tiles, 0);
    g.n_steps.assign(g.n_tiles, 0);
    g.offsets.assign(g.n_tiles, 0);
    const size_t max_samples = (size_t)g.n_tiles * NT * Cache::PADDED_BRICK_SIZE;
    g.pos.resize(max_samples);
    g.dir.resize(max_samples);
    g.t0.resize(max_samples);
    const size_t n_brick_cells = (size_t)g.bricks.x * g.bricks.y * g.bricks.z;
    g.packed.assign(n_brick_cells, -1); /* Cache::setDataArraysZero: packed index -1, data arrays 0 (src/cache.cu:13-57) */
    /* the reference indexes brick_isset_array with tiles' depth bricks also beyond the frustum depth (a camera
     * outside the scene box); four times the array's size absorbs such writes, rcb_finish counts them */
    g.isset_bricks.assign(4 * n_brick_cells, 0);
    const int3 dd = make_int3(g.data_bricks.x * Cache::PADDED_BRICK_SIZE, g.data_bricks.y * Cache::PADDED_BRICK_SIZE,
                              g.data_bricks.z * Cache::PADDED_BRICK_SIZE);
    const size_t n_vox = (size_t)dd.x * dd.y * dd.z;
    g.isset.assign(n_vox, 0.f);
    g.density.assign(n_vox, 0.f);
    for (auto &l : g.lat) l.assign(n_vox, make_ushort4(0, 0, 0, 0));
    g.known.assign((size_t)g.frustum.x * g.frustum.y, 0.f);
    g.image.assign((size_t)g.frustum.x * g.frustum.y, make_uchar4(0, 0, 0, 0));
    g_oob = 0;
    launch(g.n_tiles, g.tiles_x, [] {
        initPayloads_cache_init_kernel<Cache::BRICK_SIZE, Cache::BRICK_PADDING>(g.rm, g.scene, g.frustum, g.bricks, g.blocks.data(),
                                                                                g.rays.data(), g.alive.data());
    });
    return g.n_tiles;
}

/* the frustum's dimensions (resizeCache): W, H, depth; and its bricks */
void rcb_dims(int *out)
{
    out[0] = g.frustum.x; out[1] = g.frustum.y; out[2] = g.frustum.z;
    out[3] = g.bricks.x; out[4] = g.bricks.y; out[5] = g.bricks.z;
}

/* One sub-iteration up to the network: the exclusive sum of the alive
 * blocks, sample_cache_init_first_kernel, the sum and exclusive sum of the
 * per-block sample counts, sample_cache_init_second_kernel.  Returns the
 * iteration's sample count (0: the build is finished) and points pos / t0
 * at its samples (contracted positions, float3 each; t0). */
int rcb_search(const float **pos, const float **t0)
{
    int run = 0;
    for (int b = 0; b < g.n_tiles; ++b) { g.alive_idx[b] = run; run += g.alive[b]; }
    g.n_alive_blocks = run;
    if (run == 0) return 0;
    launch(g.n_tiles, g.n_tiles, [] {
        sample_cache_init_first_kernel<Cache::BRICK_SIZE, Cache::BRICK_PADDING>(g.rm, g.scene, g.bits.data(), g.frustum, g.bricks,
                                                                                g.blocks.data(), g.rays.data(), g.alive_idx.data(),
                                                                                g.compact.data(), g.alive.data(), g.n_steps.data());
    });
    int total = 0;
    for (int b = 0; b < g.n_alive_blocks; ++b) { g.offsets[b] = total; total += g.n_steps[b]; }
    g.n_samples = total;
    launch(g.n_alive_blocks, g.n_alive_blocks, [] {
        sample_cache_init_second_kernel<Cache::BRICK_SIZE, Cache::BRICK_PADDING>(
            g.rm, g.scene, g.bits.data(), g.frustum, g.bricks, g.n_tiles, g.blocks.data(), g.rays.data(), &g.counter, g.pos.data(),
            g.dir.data(), g.t0.data(), g.compact.data(), g.alive.data(), g.n_steps.data(), g.offsets.data());
    });
    *pos = reinterpret_cast<const float *>(g.pos.data());
    *t0 = g.t0.data();
    return total;
}

/* accumulateNew_cache_init_second_kernel on the caller's network outputs:
 * fp16 bits, row-major [n_out][batch] (row 0 the log-density). */
int rcb_accumulate(const uint16_t *network_output, int batch)
{
    if (batch < g.n_samples) return -1;
    const cudaSurfaceObject_t s_packed = reg(0, g.packed.data(), sizeof(int), g.bricks.x, g.bricks.y, g.bricks.z);
    const int3 dd = make_int3(g.data_bricks.x * Cache::PADDED_BRICK_SIZE, g.data_bricks.y * Cache::PADDED_BRICK_SIZE,
                              g.data_bricks.z * Cache::PADDED_BRICK_SIZE);
    Cache::Surfaces surf;
    surf.data_isset_surf = reg(1, g.isset.data(), sizeof(float), dd.x, dd.y, dd.z);
    surf.data_density_alpha_surf = reg(2, g.density.data(), sizeof(float), dd.x, dd.y, dd.z);
    for (int i = 0; i < Cache::N_DATA_ARRAYS; ++i) surf.data_surf[i] = reg(3 + i, g.lat[i].data(), sizeof(ushort4), dd.x, dd.y, dd.z);
    const half *out = reinterpret_cast<const half *>(network_output);
    launch(g.n_alive_blocks, g.n_alive_blocks, [&] {
        accumulateNew_cache_init_second_kernel<Cache::BRICK_SIZE, Cache::BRICK_PADDING>(
            g.rm, g.scene, g.settings, g.frustum, g.bricks, g.total_bricks, g.blocks.data(), g.rays.data(), batch, g.latent_offset,
            out, g.t0.data(), &g.counter, g.compact.data(), g.alive.data(), g.n_steps.data(), g.offsets.data(), s_packed,
            g.isset_bricks.data(), dd, g.data_bricks, surf);
    });
    return 0;
}

/* writeImageBuffer_cache_init_kernel2 (known ranges), then the results:
 * packed [bZ][bY][bX] (the reference's slots, -1 without), known ranges
 * [H][W], the count of out-of-range surface writes; returns the slot
 * counter (bricks demanded). */
int rcb_finish(int32_t *packed, float *known, long long *out_of_range)
{
    const cudaSurfaceObject_t s_known = reg(6, g.known.data(), sizeof(float), g.frustum.x, g.frustum.y, 1);
    const cudaSurfaceObject_t s_img = reg(7, g.image.data(), sizeof(uchar4), g.frustum.x, g.frustum.y, 1);
    const int2 res = make_int2(g.rm.cam_info.resolution.x, g.rm.cam_info.resolution.y);
    launch(g.n_tiles, g.tiles_x, [&] {
        writeImageBuffer_cache_init_kernel2<Cache::BRICK_SIZE, Cache::BRICK_PADDING>(res, g.bricks, g.rm, g.blocks.data(), g.rays.data(),
                                                                                     s_known, s_img);
    });
    memcpy(packed, g.packed.data(), g.packed.size() * sizeof(int));
    memcpy(known, g.known.data(), g.known.size() * sizeof(float));
    long long beyond = 0;
    for (size_t i = g.packed.size(); i < g.isset_bricks.size(); ++i) beyond += g.isset_bricks[i] != 0;
    *out_of_range = g_oob.load() + beyond;
    return g.counter;
}

/* The voxels of every frustum brick that holds a slot, in brick-cell order
 * ([bZ][bY][bX] with packed >= 0), each brick's 512 voxels [z][y][x]:
 * isset, density slot, 8 fp16 latents.  Returns the number of bricks. */
int rcb_bricks(float *isset, float *density, uint16_t *latents)
{
    const int3 dd = make_int3(g.data_bricks.x * Cache::PADDED_BRICK_SIZE, g.data_bricks.y * Cache::PADDED_BRICK_SIZE,
                              g.data_bricks.z * Cache::PADDED_BRICK_SIZE);
    int n = 0;
    for (size_t c = 0; c < g.packed.size(); ++c) {
        if (g.packed[c] < 0) continue;
        const int3 b = unpack3D(g.packed[c]);
        for (int z = 0; z < 8; ++z)
            for (int y = 0; y < 8; ++y)
                for (int x = 0; x < 8; ++x) {
                    const size_t v = ((size_t)(b.z * 8 + z) * dd.y + (b.y * 8 + y)) * dd.x + (b.x * 8 + x);
                    const size_t o = (size_t)n * 512 + (size_t)z * 64 + y * 8 + x;
                    isset[o] = g.isset[v];
                    density[o] = g.density[v];
                    for (int i = 0; i < Cache::N_DATA_ARRAYS; ++i) memcpy(latents + o * 8 + 4 * i, &g.lat[i][v], 4 * sizeof(uint16_t));
                }
        ++n;
    }
    return n;
}

} // extern "C"
