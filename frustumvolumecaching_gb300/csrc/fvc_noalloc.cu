/*
 * fvc_noalloc.cu - a plain render that allocates nothing.
 *
 * Some callers cannot call cudaMalloc while they render: a host whose GPU
 * memory is handed out by its own allocator or a fixed budget (an engine
 * plugin, a process that reserves all device memory up front), code running
 * where allocation is forbidden or too slow (per-frame callbacks with hard
 * deadlines).  fvc_render_noalloc serves them.  The caller passes the model,
 * the camera and device output buffers; the scratch the renderer needs (alive
 * ray states, the per-sub-iteration sample rows, counters) lives in one
 * file-scope device array, g_noalloc_scratch, of FVC_NOALLOC_SCRATCH_BYTES.
 * Every GPU that loads the library holds that array until the process exits.
 *
 * The array has room for FVC_NOALLOC_MAX_RAYS rays (256 x 256 pixels); larger
 * images are rejected with FVC_ERR_ARG.  All calls share the array and it
 * keeps the last call's contents, so calls whose GPU work overlaps (two
 * streams, two host threads) race on it: serialise them.  The counters that
 * must start at zero are cleared at the start of every call.
 *
 * The call blocks the host like the allocating render: every few
 * sub-iterations it reads the alive-ray count back into a host word and
 * synchronises the stream, and it returns once the frame has finished
 * marching.
 *
 * The first call on a device looks up the array's device address with
 * cudaGetSymbolAddress while that device is current; make that first call
 * before any stream capture on the device.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/fvc.h"
#include "fvc_kernels.h"

using namespace fvc;

namespace {

constexpr int ROWS_PER_RAY = 16;                 /* rows per ray and sub-iteration */
constexpr size_t BYTES_PER_RAY = 2 * sizeof(RayState) + sizeof(int2) +
                                 (size_t)ROWS_PER_RAY * (sizeof(float) + sizeof(int) + sizeof(float4) + sizeof(uint2));
constexpr size_t HEADER_BYTES = 4096;            /* counters and statistics */

}  // namespace

static_assert((size_t)FVC_NOALLOC_MAX_RAYS * BYTES_PER_RAY + HEADER_BYTES <= (size_t)FVC_NOALLOC_SCRATCH_BYTES,
              "scratch array too small for FVC_NOALLOC_MAX_RAYS");

/* The scratch: one array per device, held until the process exits. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[FVC_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_addr_mutex;
void *g_addr[256] = {};  /* device address of g_noalloc_scratch per device ordinal */

thread_local std::string g_noalloc_err;

int fail_na(int code, const std::string &msg)
{
    g_noalloc_err = msg;
    return code;
}

/* once per device, with that device current */
int scratch_address(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_na(FVC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 256) return fail_na(FVC_ERR_CUDA, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_addr_mutex);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail_na(FVC_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return FVC_OK;
}

template <class T>
T *carve(unsigned char *&cursor, size_t n)
{
    T *p = reinterpret_cast<T *>(cursor);
    cursor += (n * sizeof(T) + 255) / 256 * 256;
    return p;
}

}  // namespace

/* Model-side views and the error slot of fvc_last_error (fvc_capi.cu). */
namespace fvc_internal {
int model_views(const fvc_model *m, RenderParams *p, int *head_hidden, int *n_sms);
void set_error(const char *msg);
DevSteps steps_view(const fvc_stepsize_info &s);
DevCam cam_view(const fvc_raymarch_info &rm);
}  // namespace fvc_internal

extern "C" int fvc_render_noalloc(fvc_model *m, const fvc_raymarch_info *info, const fvc_render_outputs *out, void *cuda_stream)
{
    int rc;
    if (!m || !info) {
        fvc_internal::set_error("fvc_render_noalloc: null argument");
        return FVC_ERR_ARG;
    }
    const long long n_rays = (long long)info->cam_info.resolution.x * info->cam_info.resolution.y;
    if (info->cam_info.resolution.x <= 0 || info->cam_info.resolution.y <= 0 || n_rays > FVC_NOALLOC_MAX_RAYS) {
        const std::string msg = "fvc_render_noalloc: " + std::to_string(n_rays) + " rays exceed the scratch array's maximum of " +
                                std::to_string(FVC_NOALLOC_MAX_RAYS) + " (use fvc_render_device for larger images)";
        fvc_internal::set_error(msg.c_str());
        return FVC_ERR_ARG;
    }
    void *base = nullptr;
    if ((rc = scratch_address(&base))) {
        fvc_internal::set_error(g_noalloc_err.c_str());
        return rc;
    }
    RenderParams p;
    memset(&p, 0, sizeof(p));
    int head_hidden = 2, n_sms = 1;
    if ((rc = fvc_internal::model_views(m, &p, &head_hidden, &n_sms))) return rc;
    p.steps = fvc_internal::steps_view(info->stepsize_info);
    p.cam = fvc_internal::cam_view(*info);
    /* carve the scratch: header (counters, statistics) then per-ray arrays */
    unsigned char *cursor = static_cast<unsigned char *>(base);
    int *ctl = carve<int>(cursor, 16);              /* [0] ray counter, [1] guard, [8..15] sub-iteration counters */
    RenderStatsDev *stats = carve<RenderStatsDev>(cursor, 1);
    cursor = static_cast<unsigned char *>(base) + HEADER_BYTES;
    const size_t n = (size_t)n_rays, cap = n * ROWS_PER_RAY;
    p.states[0] = carve<RayState>(cursor, n);
    p.states[1] = carve<RayState>(cursor, n);
    p.ray_rows = carve<int2>(cursor, n);
    p.row_t0 = carve<float>(cursor, cap);
    p.row_slot = carve<int>(cursor, cap);
    p.row_pay = carve<float4>(cursor, cap);
    p.row_out = carve<uint2>(cursor, cap);
    p.counters = ctl + 8;
    p.ray_counter = ctl;
    p.guard = ctl + 1;
    p.stats = stats;
    p.row_capacity = (int)cap;
    p.steps_per_iter = 64;
    p.skip_empty = 0;
    p.results = out ? (float4 *)out->results : nullptr;
    p.image = out ? (uchar4 *)out->image_rgba8 : nullptr;
    p.ray_counts = out ? (int4 *)out->ray_counts : nullptr;
    p.sample_index = info->sample_index;
    p.max_rounds = 1 << 26;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    cudaError_t e = cudaMemsetAsync(base, 0, HEADER_BYTES, s);
    if (e == cudaSuccess) {
        int h_alive = 0; /* pageable host word: the alive-count readback needs no pinned allocation */
        e = render_frame(p, false, head_hidden, n_sms, s, &h_alive, 4, nullptr);
    }
    if (e != cudaSuccess) {
        const std::string msg = std::string("fvc_render_noalloc: ") + cudaGetErrorString(e);
        fvc_internal::set_error(msg.c_str());
        return FVC_ERR_CUDA;
    }
    return FVC_OK;
}
