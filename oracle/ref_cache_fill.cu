/*
 * ref_cache_fill.cu - runs the reference's own per-ray cache-fill kernels on
 * the host to make golden vectors.  TEST INFRASTRUCTURE ONLY (built by
 * oracle/Makefile into oracle/_ref/libref_cache_fill.so, never part of the
 * product).
 *
 * The kernels are initRayPayloads_common_kernel,
 * compactPayloads_atomic_common_kernel and sample_common_kernel
 * (src/renderer.cu:36-85,136-157,192-243), and
 * accumulate_cache_init_first_kernel, accumulate_cache_init_second_kernel,
 * reserveNewBricks_kernel and writeImageBuffer_cache_init_kernel
 * (src/cache_renderer.cu:571-830).  Their text is cut unchanged out of the
 * reference files at build time (oracle/Makefile, into oracle/_ref/) and
 * compiled here by nvcc as host functions; the reference headers come
 * unchanged through -I.  None of these kernels synchronises its block, so
 * each CUDA thread runs on the host one after another (threadIdx / blockIdx
 * set per thread); atomicAdd is then a plain add in thread order, one of the
 * orders a GPU may take; tex3D / surf3Dread / surf3Dwrite / surf2Dwrite read
 * and write host arrays registered as handles; __float2int_rd is floorf.  CacheSettings /
 * DensityInterpolVariant repeat include/cache_renderer.h:15-32, which cannot
 * be included (it pulls in tiny-cuda-nn).
 *
 * rcf_* restate the host loop of CacheRenderer::initCache
 * (src/cache_renderer.cu:848-928): compaction of the alive payloads,
 * clamp(2^21 / alive, 1, 8) samples per ray and sub-iteration, the kernels
 * around the network, the known ranges at the end.  The network
 * (NerfNetwork::inferenceLatents) is the caller's: rcf_search returns the
 * sub-iteration's sample positions, the caller writes the fp16 outputs
 * row-major [rows][batch] and calls rcf_accumulate.
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstring>
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

static uint3 g_tid, g_bid;
static dim3 g_bdim;

struct HostArray {
    void *data = nullptr;
    size_t elem = 0;
    int dx = 0, dy = 0, dz = 0;
};
static std::vector<HostArray> g_arr(8);
static long long g_oob = 0;

template <class T> static T *host_at(unsigned long long h, int x, int y, int z)
{
    HostArray &a = g_arr[(size_t)h];
    if (sizeof(T) != a.elem || x < 0 || y < 0 || z < 0 || x >= a.dx || y >= a.dy || z >= a.dz) return nullptr;
    return reinterpret_cast<T *>(a.data) + ((size_t)z * a.dy + y) * a.dx + x;
}
template <class T> static void host_surf3Dwrite(T v, cudaSurfaceObject_t s, const int3 idx)
{
    T *p = host_at<T>(s, idx.x, idx.y, idx.z);
    if (p) *p = v; else ++g_oob;
}
template <class T> static T host_surf3Dread(cudaSurfaceObject_t s, int x_bytes, int y, int z)
{
    T *p = host_at<T>(s, x_bytes / (int)sizeof(T), y, z);
    if (!p) { ++g_oob; return T(); }
    return *p;
}
template <class T> static void host_surf2Dwrite(T v, cudaSurfaceObject_t s, int x_bytes, int y)
{
    host_surf3Dwrite<T>(v, s, make_int3(x_bytes / (int)sizeof(T), y, 0));
}
/* point-sampled integer texture (border reads 0, the reference's texture address mode) */
template <class T> static T host_tex3D(cudaTextureObject_t t, int3 idx)
{
    T *p = host_at<T>(t, idx.x, idx.y, idx.z);
    return p ? *p : T();
}
static int host_atomicAdd(int *p, int v) { const int o = *p; *p += v; return o; }
/* __float2int_rd: round toward minus infinity */
static int host_float2int_rd(float x) { return (int)floorf(x); }

#undef __global__
#define __global__ static
#define threadIdx g_tid
#define blockIdx g_bid
#define blockDim g_bdim
#define surf3Dwrite host_surf3Dwrite
#define surf3Dread host_surf3Dread
#define surf2Dwrite host_surf2Dwrite
#define tex3D host_tex3D
#define atomicAdd host_atomicAdd
#define __float2int_rd host_float2int_rd
#include "cache_fill_kernels.inc"
#undef threadIdx
#undef blockIdx
#undef blockDim
#undef surf3Dwrite
#undef surf3Dread
#undef surf2Dwrite
#undef tex3D
#undef atomicAdd
#undef __float2int_rd

template <class F> static void launch1d(int n, int bs, F fn)
{
    g_bdim = dim3(bs, 1, 1);
    for (int i = 0; i < (n + bs - 1) / bs * bs; ++i) {
        g_tid = make_uint3(i % bs, 0, 0);
        g_bid = make_uint3(i / bs, 0, 0);
        fn();
    }
}
template <class F> static void launch2d(int nx, int ny, int bs, F fn)
{
    g_bdim = dim3(bs, bs, 1);
    for (int y = 0; y < (ny + bs - 1) / bs * bs; ++y)
        for (int x = 0; x < (nx + bs - 1) / bs * bs; ++x) {
            g_tid = make_uint3(x % bs, y % bs, 0);
            g_bid = make_uint3(x / bs, y / bs, 0);
            fn();
        }
}

struct Fill {
    RaymarchInfo rm;
    SceneInfo scene;
    CacheSettings settings;
    std::vector<uint8_t> bits;
    int3 frustum, bricks, data_bricks;
    int n_rays = 0, n_alive = 0, n_steps = 0, batch = 0, subiter = 0, total_bricks = 0, latent_offset = 0, counter = 0;
    std::vector<RayPayload> pay[2], fin;
    std::vector<float3> pos, dir;
    std::vector<float> t0;
    std::vector<char> isset_sub, isset_bricks;
    std::vector<int> brick_index, packed;
    std::vector<float> isset, density, known;
    std::vector<ushort4> lat[Cache::N_DATA_ARRAYS];
    std::vector<uchar4> image;
};
static Fill g;

extern "C" {

/* Set-up (the parameters as rcb_init's in ref_cache_build.cu) and
 * initRayPayloads_common_kernel.  Returns the number of rays. */
int rcf_init(const int *sc, const float *f, int W, int H, const uint8_t *bits, const int *data_bricks, int latent_offset, int variant)
{
    g = Fill();
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
    const int max_n_steps = (int)ceil(max_step_in_scene(st, si)); /* resizeCache, src/cache_renderer.cu:832-846 */
    g.frustum = make_int3(W, H, (max_n_steps + 3) / 4 * 4);
    g.bricks = make_int3((g.frustum.x + 7) / 8, (g.frustum.y + 7) / 8, (g.frustum.z + 7) / 8);
    g.data_bricks = make_int3(data_bricks[0], data_bricks[1], data_bricks[2]);
    g.total_bricks = data_bricks[0] * data_bricks[1] * data_bricks[2];
    g.latent_offset = latent_offset;
    g.n_rays = g.n_alive = W * H;
    for (auto &p : g.pay) p.assign(g.n_rays, RayPayload{});
    g.fin.assign(g.n_rays, RayPayload{});
    g.pos.assign((size_t)g.n_rays * 8, make_float3(0.f, 0.f, 0.f));
    g.dir.assign((size_t)g.n_rays * 8, make_float3(0.f, 0.f, 0.f));
    g.t0.assign((size_t)g.n_rays * 8, 0.f);
    const size_t cells = (size_t)g.bricks.x * g.bricks.y * g.bricks.z;
    g.isset_sub.assign(cells, 0); /* Cache::setDataArraysZero (src/cache.cu:13-57) */
    g.isset_bricks.assign(cells, 0);
    g.brick_index.assign(cells, 0);
    g.packed.assign(cells, -1);
    const int3 dd = make_int3(g.data_bricks.x * 8, g.data_bricks.y * 8, g.data_bricks.z * 8);
    const size_t nv = (size_t)dd.x * dd.y * dd.z;
    g.isset.assign(nv, 0.f);
    g.density.assign(nv, 0.f);
    for (auto &l : g.lat) l.assign(nv, make_ushort4(0, 0, 0, 0));
    g.known.assign((size_t)W * H, 0.f);
    g.image.assign((size_t)W * H, make_uchar4(0, 0, 0, 0));
    g_arr[0] = HostArray{g.packed.data(), sizeof(int), g.bricks.x, g.bricks.y, g.bricks.z};
    g_arr[1] = HostArray{g.isset.data(), sizeof(float), dd.x, dd.y, dd.z};
    g_arr[2] = HostArray{g.density.data(), sizeof(float), dd.x, dd.y, dd.z};
    for (int i = 0; i < Cache::N_DATA_ARRAYS; ++i) g_arr[3 + i] = HostArray{g.lat[i].data(), sizeof(ushort4), dd.x, dd.y, dd.z};
    g_arr[6] = HostArray{g.known.data(), sizeof(float), W, H, 1};
    g_arr[7] = HostArray{g.image.data(), sizeof(uchar4), W, H, 1};
    g_oob = 0;
    launch2d(W, H, 16, [] { initRayPayloads_common_kernel(g.rm, g.scene, g.pay[0].data(), nullptr); });
    return g.n_rays;
}

/* One sub-iteration up to the network: compaction, then sample_common_kernel
 * with clamp(2^21 / alive, 1, 8) samples per ray.  Returns the rows of the
 * batch (alive * samples per ray, row = step * alive + ray; 0: finished) and
 * points pos (float3 per row; rows a ray did not fill read as zero) at them;
 * *batch receives next_multiple(rows, 256). */
int rcf_search(const float **pos, int *batch)
{
    std::vector<RayPayload> &prev = g.pay[g.subiter % 2], &curr = g.pay[(g.subiter + 1) % 2];
    std::fill(g.isset_sub.begin(), g.isset_sub.end(), 0);
    int counter = 0;
    launch1d(g.n_alive, 128, [&] { compactPayloads_atomic_common_kernel(g.n_alive, prev.data(), curr.data(), g.fin.data(), &counter); });
    g.n_alive = counter;
    if (g.n_alive == 0) return 0;
    g.n_steps = std::min(8, std::max(1, (1 << 21) / g.n_alive)); /* TARGET_BATCH_SIZE, MIN/MAX_N_STEPS_PER_SUBITER */
    const int rows = g.n_alive * g.n_steps;
    g.batch = (rows + 255) / 256 * 256;
    std::fill(g.pos.begin(), g.pos.begin() + rows, make_float3(0.f, 0.f, 0.f));
    launch1d(g.n_alive, 128, [&] {
        sample_common_kernel(g.n_alive, g.n_steps, g.rm, g.scene, g.bits.data(), curr.data(), g.pos.data(), g.dir.data(), g.t0.data());
    });
    *pos = reinterpret_cast<const float *>(g.pos.data());
    *batch = g.batch;
    return rows;
}

/* The kernels after the network on its fp16 outputs (row-major [n_out][batch]). */
int rcf_accumulate(const uint16_t *network_output)
{
    std::vector<RayPayload> &curr = g.pay[(g.subiter + 1) % 2];
    const half *out = reinterpret_cast<const half *>(network_output);
    launch1d(g.n_alive, 128, [&] {
        accumulate_cache_init_first_kernel(g.n_alive, g.batch, g.rm, g.scene, curr.data(), out, g.t0.data(), g.frustum, g.bricks,
                                           g.isset_sub.data());
    });
    launch2d(g.bricks.x, g.bricks.y, 16, [&] {
        reserveNewBricks_kernel(g.bricks, g.data_bricks, g.total_bricks, &g.counter, g.isset_sub.data(), g.isset_bricks.data(),
                                g.brick_index.data(), (cudaSurfaceObject_t)0);
    });
    Cache::Surfaces surf;
    surf.data_isset_surf = 1;
    surf.data_density_alpha_surf = 2;
    for (int i = 0; i < Cache::N_DATA_ARRAYS; ++i) surf.data_surf[i] = 3 + i;
    const int3 dd = make_int3(g.data_bricks.x * 8, g.data_bricks.y * 8, g.data_bricks.z * 8);
    launch1d(g.n_alive, 128, [&] {
        accumulate_cache_init_second_kernel(g.n_alive, g.batch, g.rm, g.scene, g.settings, curr.data(), out, g.latent_offset, g.t0.data(),
                                            g.frustum, g.bricks, g.isset_sub.data(), g.brick_index.data(), (cudaTextureObject_t)0, dd,
                                            g.data_bricks, surf);
    });
    ++g.subiter;
    return 0;
}

/* writeImageBuffer_cache_init_kernel (known ranges) and the results as
 * rcb_finish / rcb_bricks of ref_cache_build.cu. */
int rcf_finish(int32_t *packed, float *known, long long *out_of_range)
{
    const int W = g.rm.cam_info.resolution.x, H = g.rm.cam_info.resolution.y;
    launch2d(W, H, 16, [&] {
        writeImageBuffer_cache_init_kernel(make_int2(W, H), g.fin.data(), (cudaSurfaceObject_t)6, (cudaSurfaceObject_t)7);
    });
    memcpy(packed, g.packed.data(), g.packed.size() * sizeof(int));
    memcpy(known, g.known.data(), g.known.size() * sizeof(float));
    *out_of_range = g_oob;
    return g.counter;
}

void rcf_dims(int *out)
{
    out[0] = g.frustum.x; out[1] = g.frustum.y; out[2] = g.frustum.z;
    out[3] = g.bricks.x; out[4] = g.bricks.y; out[5] = g.bricks.z;
}

int rcf_bricks(float *isset, float *density, uint16_t *latents)
{
    const int3 dd = make_int3(g.data_bricks.x * 8, g.data_bricks.y * 8, g.data_bricks.z * 8);
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
