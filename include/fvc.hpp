/*
 * fvc.hpp - the reference's C++ renderer API, implemented over the C ABI of
 * fvc.h (header-only; link libfvc.so and the CUDA runtime).
 *
 * A caller of the reference includes this header instead of the reference's
 * renderer headers and keeps its code: the same type names and field layouts
 * (include/common.h:22-218), the same loader entry points (include/loader.h:
 * 32-51), the same renderer classes and members (include/renderer.h:77-119,
 * basic_renderer.h, performance_renderer.h:19-64, cache_renderer.h:34-109,
 * cache_performance_renderer.h:21-131, cache_basic_renderer.h:10-40) and the
 * same error behaviour
 * (std::runtime_error; loaders return false).  Renders are synchronous like
 * the reference's.
 *
 * Differences a caller can see:
 *  - NerfNetwork is a handle to the model inside libfvc.so (no tcnn objects);
 *  - RenderBuffer is a headless device buffer (uchar4 image + float4 rgb/T)
 *    instead of a CUDA surface, and writeToFile writes PNG only;
 *  - cache brick slots are assigned in a fixed order (the reference uses
 *    atomicAdd), so builds are reproducible;
 *  - DebugData contribution buffers are accepted and left untouched;
 *  - Renderer::_timer records whole-render wall time and the event-timed
 *    resample network kernel, not the reference's nine phases.
 */
#pragma once

#include "fvc.h"

#include <cuda_fp16.h>
#include <cuda_runtime_api.h>
#include <vector_types.h>

#include <algorithm>
#include <functional>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace fs = std::filesystem;

/* ------------------------------------------------------------------------ */
/* errors                                                                    */
/* ------------------------------------------------------------------------ */
namespace fvc_cpp {
inline void check(int rc)
{
    if (rc != FVC_OK) throw std::runtime_error(fvc_last_error());
}
inline void check_cuda(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace fvc_cpp

/* ------------------------------------------------------------------------ */
/* POD types with the reference's layouts                                    */
/* ------------------------------------------------------------------------ */

/* CameraMatrix, include/common.h:22-62: rows of a 3x4 [R|t]. */
struct CameraMatrix {
    float4 m0, m1, m2;

    /* the rigid inverse [R^T | -R^T t] */
    CameraMatrix inverse() const
    {
        const float c0[3] = {m0.x, m1.x, m2.x}, c1[3] = {m0.y, m1.y, m2.y}, c2[3] = {m0.z, m1.z, m2.z};
        const float t[3] = {m0.w, m1.w, m2.w};
        auto dot3 = [](const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
        return {make_float4(c0[0], c0[1], c0[2], -dot3(c0, t)), make_float4(c1[0], c1[1], c1[2], -dot3(c1, t)),
                make_float4(c2[0], c2[1], c2[2], -dot3(c2, t))};
    }
    float3 getTranslation() const { return make_float3(m0.w, m1.w, m2.w); }
};

enum ContractionType { NONE = 0, AABB = 1, WARP_AABB_L2 = 2, WARP_AABB_LINF = 3 };

/* SceneInfo, include/common.h:74-91. */
struct SceneInfo {
    int grid_resolution;
    int grid_nlvl;
    int vals_per_lvl;
    bool normalized;
    float3 aabb_from, aabb_to;
    float3 contraction_aabb_from, contraction_aabb_to;
    int contraction_type;
    bool is_open_gl;
    float alpha_thre;
};

struct SceneInfo;

/* StepsizeInfo, include/common.h:93-164 (the derived fields are filled by the
 * loader, or by setAdditionalInfo). */
struct StepsizeInfo {
    float cone_angle, log1p_c, stepsize, near, near_i, far;
    float dt_min, dt_max, t_min, t_max, i_min, i_max;

    inline void setAdditionalInfo(const SceneInfo &scene_info);
    void changeSamplingRate(const float factor, const SceneInfo &scene_info)
    {
        cone_angle /= factor;
        stepsize /= factor;
        setAdditionalInfo(scene_info);
    }
};

/* CameraInfo, include/common.h:166-195. */
struct CameraInfo {
    int2 resolution;
    bool is_open_gl;
    float2 focal;
    float2 principal;
    CameraMatrix cam2world;
    CameraMatrix world2cam;
    float aperature = 0.0f;
    float focus_z = 1.0f;

    /* keeps the vertical field of view (include/common.h:180-185) */
    void resize(int2 r)
    {
        const float s = r.y / (float)resolution.y;
        focal = make_float2(s * focal.x, s * focal.y);
        principal = make_float2(principal.x * r.x / (float)resolution.x, principal.y * r.y / (float)resolution.y);
        resolution = r;
    }
    CameraInfo createUpdated(CameraMatrix &c2w, int2 r) const
    {
        CameraInfo n = *this;
        n.cam2world = c2w;
        n.world2cam = c2w.inverse();
        n.resize(r);
        return n;
    }
};

/* RaymarchInfo, include/common.h:210-218. */
struct RaymarchInfo {
    CameraInfo cam_info;
    CameraInfo next_cam_info;
    StepsizeInfo stepsize_info;
    int sample_index;
    bool motion_blur;
    bool deterministic;
};

/* CameraPathDataEntry, include/common.h:204-208. */
struct CameraPathDataEntry {
    CameraMatrix transform_matrix;
    fs::path image_path;
};

static_assert(sizeof(SceneInfo) == sizeof(fvc_scene_info) && offsetof(SceneInfo, aabb_from) == offsetof(fvc_scene_info, aabb_from) &&
                  offsetof(SceneInfo, alpha_thre) == offsetof(fvc_scene_info, alpha_thre), "SceneInfo layout");
static_assert(sizeof(StepsizeInfo) == sizeof(fvc_stepsize_info), "StepsizeInfo layout");
static_assert(sizeof(CameraInfo) == sizeof(fvc_camera_info) && offsetof(CameraInfo, focal) == offsetof(fvc_camera_info, focal) &&
                  offsetof(CameraInfo, cam2world) == offsetof(fvc_camera_info, cam2world) &&
                  offsetof(CameraInfo, focus_z) == offsetof(fvc_camera_info, focus_z), "CameraInfo layout");
static_assert(sizeof(RaymarchInfo) == sizeof(fvc_raymarch_info) &&
                  offsetof(RaymarchInfo, stepsize_info) == offsetof(fvc_raymarch_info, stepsize_info) &&
                  offsetof(RaymarchInfo, deterministic) == offsetof(fvc_raymarch_info, deterministic), "RaymarchInfo layout");

namespace fvc_cpp {
inline const fvc_raymarch_info *abi(const RaymarchInfo &r) { return reinterpret_cast<const fvc_raymarch_info *>(&r); }
inline const fvc_stepsize_info *abi(const StepsizeInfo &s) { return reinterpret_cast<const fvc_stepsize_info *>(&s); }
inline const fvc_scene_info *abi(const SceneInfo &s) { return reinterpret_cast<const fvc_scene_info *>(&s); }
}  // namespace fvc_cpp

inline void StepsizeInfo::setAdditionalInfo(const SceneInfo &scene_info)
{
    fvc_cpp::check(fvc_stepsize_setup(fvc_cpp::abi(scene_info), reinterpret_cast<fvc_stepsize_info *>(this)));
}

/* ------------------------------------------------------------------------ */
/* device memory                                                             */
/* ------------------------------------------------------------------------ */

/* CudaBuffer<T>, include/util/buffer.h: an owning device array, or (for the
 * loader's occupancy grid) a view of memory owned by the model. */
template <typename T>
class CudaBuffer {
public:
    CudaBuffer() = default;
    explicit CudaBuffer(size_t n) { resize(n); }
    CudaBuffer(const CudaBuffer &) = delete;
    CudaBuffer &operator=(const CudaBuffer &) = delete;
    ~CudaBuffer() { release(); }

    static CudaBuffer view(const T *p, size_t n)
    {
        CudaBuffer b;
        b._ptr = const_cast<T *>(p);
        b._size = n;
        b._owned = false;
        return b;
    }
    CudaBuffer(CudaBuffer &&o) noexcept : _ptr(o._ptr), _size(o._size), _owned(o._owned) { o._ptr = nullptr; o._size = 0; }
    CudaBuffer &operator=(CudaBuffer &&o) noexcept
    {
        if (this != &o) {
            release();
            _ptr = o._ptr; _size = o._size; _owned = o._owned;
            o._ptr = nullptr; o._size = 0;
        }
        return *this;
    }
    void resize(size_t n)
    {
        if (n == _size && _owned) return;
        release();
        if (n) fvc_cpp::check_cuda(cudaMalloc((void **)&_ptr, n * sizeof(T)), "CudaBuffer::resize");
        _size = n;
        _owned = true;
    }
    void upload(const T *h) { fvc_cpp::check_cuda(cudaMemcpy(_ptr, h, _size * sizeof(T), cudaMemcpyHostToDevice), "upload"); }
    void download(T *h) const { fvc_cpp::check_cuda(cudaMemcpy(h, _ptr, _size * sizeof(T), cudaMemcpyDeviceToHost), "download"); }
    void download(std::vector<T> &h) const { h.resize(_size); download(h.data()); }
    void memset(int v) { fvc_cpp::check_cuda(cudaMemset(_ptr, v, _size * sizeof(T)), "memset"); }
    T *data() { return _ptr; }
    const T *data() const { return _ptr; }
    size_t size() const { return _size; }
    size_t bytesize() const { return _size * sizeof(T); }

private:
    void release()
    {
        if (_ptr && _owned) cudaFree(_ptr);
        _ptr = nullptr;
        _size = 0;
    }
    T *_ptr = nullptr;
    size_t _size = 0;
    bool _owned = true;
};

/* ------------------------------------------------------------------------ */
/* PNG output and JSON input (self-contained; no third-party libraries)      */
/* ------------------------------------------------------------------------ */
namespace fvc_cpp {

inline uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0)
{
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1u) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            table[i] = v;
        }
        init = true;
    }
    c = ~c;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return ~c;
}

/* 8-bit PNG (channels 4: RGBA, 1: gray) with uncompressed (stored) deflate blocks */
inline bool write_png(const fs::path &path, const uint8_t *rgba, int w, int h, int channels = 4)
{
    std::vector<uint8_t> raw;
    const size_t row = (size_t)w * channels;
    raw.reserve((size_t)h * (1 + row));
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba + (size_t)y * row, rgba + (size_t)(y + 1) * row);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    uint32_t a = 1, b = 0;
    for (uint8_t v : raw) { a = (a + v) % 65521u; b = (b + a) % 65521u; }
    for (size_t off = 0; off < raw.size() || off == 0; off += 65535) {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        z.push_back(off + len >= raw.size() ? 1 : 0);
        z.push_back(len & 0xFF); z.push_back(len >> 8);
        z.push_back(~len & 0xFF); z.push_back((~len >> 8) & 0xFF);
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        if (raw.empty()) break;
    }
    const uint32_t adler = (b << 16) | a;
    for (int s = 24; s >= 0; s -= 8) z.push_back((adler >> s) & 0xFF);
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    auto be32 = [&](uint32_t v) { uint8_t q[4] = {uint8_t(v >> 24), uint8_t(v >> 16), uint8_t(v >> 8), uint8_t(v)}; f.write((char *)q, 4); };
    auto chunk = [&](const char *type, const std::vector<uint8_t> &d) {
        be32((uint32_t)d.size());
        std::vector<uint8_t> td(type, type + 4);
        td.insert(td.end(), d.begin(), d.end());
        f.write((const char *)td.data(), td.size());
        be32(crc32(td.data(), td.size()));
    };
    const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    f.write((const char *)sig, 8);
    std::vector<uint8_t> ihdr(13);
    for (int i = 0; i < 4; ++i) { ihdr[i] = uint8_t(w >> (24 - 8 * i)); ihdr[4 + i] = uint8_t(h >> (24 - 8 * i)); }
    ihdr[8] = 8; ihdr[9] = channels == 1 ? 0 : 6; ihdr[10] = ihdr[11] = ihdr[12] = 0;
    chunk("IHDR", ihdr);
    chunk("IDAT", z);
    chunk("IEND", {});
    return (bool)f;
}

/* minimal JSON value and recursive-descent reader */
struct Json {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    double num = 0;
    bool b = false;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;
    bool contains(const std::string &k) const { return kind == OBJ && obj.count(k); }
    const Json &operator[](const std::string &k) const
    {
        auto it = obj.find(k);
        if (it == obj.end()) throw std::runtime_error("json: missing key " + k);
        return it->second;
    }
    const Json &operator[](size_t i) const
    {
        if (kind != ARR || i >= arr.size()) throw std::runtime_error("json: index out of range");
        return arr[i];
    }
    float f() const
    {
        if (kind != NUM) throw std::runtime_error("json: number expected");
        return (float)num;
    }
};

inline Json parse_json(const char *&p, const char *e)
{
    auto ws = [&]() { while (p < e && std::isspace((unsigned char)*p)) ++p; };
    ws();
    Json v;
    if (p >= e) throw std::runtime_error("json: unexpected end");
    if (*p == '{' || *p == '[') {
        const bool obj = *p == '{';
        v.kind = obj ? Json::OBJ : Json::ARR;
        ++p; ws();
        if (p < e && *p == (obj ? '}' : ']')) { ++p; return v; }
        for (;;) {
            if (obj) {
                Json k = parse_json(p, e);
                if (k.kind != Json::STR) throw std::runtime_error("json: key expected");
                ws();
                if (p >= e || *p != ':') throw std::runtime_error("json: ':' expected");
                ++p;
                v.obj[k.str] = parse_json(p, e);
            } else {
                v.arr.push_back(parse_json(p, e));
            }
            ws();
            if (p < e && *p == ',') { ++p; continue; }
            if (p < e && *p == (obj ? '}' : ']')) { ++p; break; }
            throw std::runtime_error("json: ',' expected");
        }
    } else if (*p == '"') {
        v.kind = Json::STR;
        ++p;
        while (p < e && *p != '"') {
            if (*p == '\\' && p + 1 < e) {
                ++p;
                v.str.push_back(*p == 'n' ? '\n' : *p == 't' ? '\t' : *p);
                ++p;
            } else {
                v.str.push_back(*p++);
            }
        }
        if (p >= e) throw std::runtime_error("json: unterminated string");
        ++p;
    } else if (e - p >= 4 && !std::strncmp(p, "true", 4)) { p += 4; v.kind = Json::BOOL; v.b = true; }
    else if (e - p >= 5 && !std::strncmp(p, "false", 5)) { p += 5; v.kind = Json::BOOL; }
    else if (e - p >= 4 && !std::strncmp(p, "null", 4)) { p += 4; }
    else {
        char *end = nullptr;
        v.num = std::strtod(p, &end);
        if (end == p) throw std::runtime_error("json: bad value");
        v.kind = Json::NUM;
        p = end;
    }
    return v;
}

inline Json read_json(const fs::path &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path.string());
    std::string s((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    const char *p = s.data();
    return parse_json(p, s.data() + s.size());
}

}  // namespace fvc_cpp

/* ------------------------------------------------------------------------ */
/* model and loader                                                          */
/* ------------------------------------------------------------------------ */

/* NerfNetwork<half>, include/nerf_network.h: here a handle to the model that
 * libfvc.so loaded (hash grid, density MLP, color head). */
template <typename T>
struct NerfNetwork {
    fvc_model *_model = nullptr;
    bool m_first_latent_is_density = false;
    int m_head_hidden_layers = 2;
    int latent_offset() const { return m_first_latent_is_density ? 0 : 1; }
};

enum DataSource { INGP = 0, NERFACC = 1 };

inline std::string dataSourceSuffix(DataSource d) { return d == INGP ? "ingp" : d == NERFACC ? "nerfacc" : "unknown"; }

/* LoaderData, include/loader.h:32-47 (owns the model). */
struct LoaderData {
    DataSource data_source = NERFACC;
    SceneInfo scene_info{};
    StepsizeInfo stepsize_info{};
    NerfNetwork<half> nerf_network;
    CudaBuffer<uint8_t> occupancy_grid_morton_bitfield;

    LoaderData() = default;
    LoaderData(const LoaderData &) = delete;
    LoaderData &operator=(const LoaderData &) = delete;
    ~LoaderData()
    {
        occupancy_grid_morton_bitfield = CudaBuffer<uint8_t>();
        if (nerf_network._model) fvc_model_destroy(nerf_network._model);
    }
};

/* load_data(fs::path, LoaderData&), src/loader.cu:287-300: an instant-ngp
 * snapshot (extension .ingp) or a nerfacc export directory (config.json +
 * tables/weights/occupancy).  Prints the reason and returns false on failure. */
inline bool load_data(fs::path data_dir, LoaderData &d)
{
    fvc_model *m = nullptr;
    if (fvc_model_load(data_dir.string().c_str(), &m) != FVC_OK) {
        std::cout << fvc_last_error() << std::endl;
        return false;
    }
    if (d.nerf_network._model) fvc_model_destroy(d.nerf_network._model);
    fvc_model_props props{};
    fvc_model_info(m, reinterpret_cast<fvc_scene_info *>(&d.scene_info), reinterpret_cast<fvc_stepsize_info *>(&d.stepsize_info));
    fvc_model_properties(m, &props);
    d.data_source = data_dir.extension() == fs::path(".ingp") ? INGP : NERFACC;
    d.nerf_network._model = m;
    d.nerf_network.m_first_latent_is_density = props.first_latent_is_density != 0;
    d.nerf_network.m_head_hidden_layers = props.head_hidden_layers;
    d.occupancy_grid_morton_bitfield = CudaBuffer<uint8_t>::view(props.occupancy_bitfield, props.occupancy_bytes);
    return true;
}

/* load_camerapath, src/loader.cu:322-378: the nerfacc camera file (width,
 * height, is_open_gl, 3x3 intrinsics, frames[].transform_matrix rows and
 * image_path) or the instant-ngp one (w/h, fl_x/fl_y/cx/cy or camera_angle_x,
 * frames[].file_path, matrices converted by nerf_matrix_to_ngp). */
inline bool load_camerapath(fs::path file, DataSource source, CameraInfo &ci, std::vector<CameraPathDataEntry> &path)
{
    using fvc_cpp::Json;
    Json j;
    try {
        j = fvc_cpp::read_json(file);
    } catch (const std::exception &) {
        std::cout << "Could not load camera path file!" << std::endl;
        return false;
    }
    auto matrix = [](const Json &m) {
        CameraMatrix c;
        c.m0 = make_float4(m[0][0].f(), m[0][1].f(), m[0][2].f(), m[0][3].f());
        c.m1 = make_float4(m[1][0].f(), m[1][1].f(), m[1][2].f(), m[1][3].f());
        c.m2 = make_float4(m[2][0].f(), m[2][1].f(), m[2][2].f(), m[2][3].f());
        return c;
    };
    auto with_ext = [](fs::path p) {
        if (!p.has_extension()) p.replace_extension(".png");
        return p;
    };
    if (source == NERFACC) {
        ci.resolution = make_int2((int)j["width"].num, (int)j["height"].num);
        ci.is_open_gl = j["is_open_gl"].b;
        const Json &K = j["intrinsics"];
        ci.focal = make_float2(K[0][0].f(), K[1][1].f());
        ci.principal = make_float2(K[0][2].f(), K[1][2].f());
        for (const Json &fr : j["frames"].arr) path.push_back({matrix(fr["transform_matrix"]), with_ext(fr["image_path"].str)});
    } else {
        const int w = j.contains("w") ? (int)j["w"].num : 800, h = j.contains("h") ? (int)j["h"].num : 800;
        ci.resolution = make_int2(w, h);
        ci.is_open_gl = false;
        if (j.contains("fl_x")) {
            ci.focal = make_float2(j["fl_x"].f(), j["fl_y"].f());
            ci.principal = make_float2(j["cx"].f(), j["cy"].f());
        } else if (j.contains("camera_angle_x")) {
            const float f = 0.5f * (float)w / std::tan(0.5f * j["camera_angle_x"].f());
            ci.focal = make_float2(f, f);
            ci.principal = make_float2(0.5f * w, 0.5f * h);
        } else {
            throw std::runtime_error("Unknown Camera Info file source");
        }
        for (const Json &fr : j["frames"].arr) {
            CameraMatrix m = matrix(fr["transform_matrix"]);
            /* scale (1,-1,-1), translation * 0.33 + 0.5, then rows cycled (y,z,x) */
            auto conv = [](float4 r) { return make_float4(r.x, -r.y, -r.z, r.w * 0.33f + 0.5f); };
            const float4 r0 = conv(m.m0), r1 = conv(m.m1), r2 = conv(m.m2);
            m.m0 = r1; m.m1 = r2; m.m2 = r0;
            path.push_back({m, with_ext(fr["file_path"].str)});
        }
    }
    ci.aperature = 0.0f;
    ci.focus_z = 1.0f;
    std::cout << "Loaded " << path.size() << " camera path frames" << std::endl;
    return true;
}

/* ------------------------------------------------------------------------ */
/* render targets                                                            */
/* ------------------------------------------------------------------------ */

/* RenderBuffer, include/util/buffer.h:165-175: a headless device target. */
struct RenderBuffer {
    virtual ~RenderBuffer() = default;
    virtual int2 resolution() const = 0;
    virtual uchar4 *image_device() = 0;
    virtual float4 *results_device() = 0;
};

/* ImageBuffer, include/util/image_buffer.h:15-41: uchar4 image (white
 * background, as the reference's writeImageBuffer kernels) + float4 rgb/T. */
class ImageBuffer : public RenderBuffer {
public:
    explicit ImageBuffer(int2 r) { resize(r); }
    void resize(int2 r)
    {
        _res = r;
        _img.resize((size_t)r.x * r.y);
        _rgbt.resize((size_t)r.x * r.y);
        _img.memset(0);
        _rgbt.memset(0);
    }
    int2 resolution() const override { return _res; }
    uchar4 *image_device() override { return _img.data(); }
    float4 *results_device() override { return _rgbt.data(); }

    std::vector<uchar4> download() const
    {
        std::vector<uchar4> h;
        _img.download(h);
        return h;
    }
    void upload(const std::vector<uchar4> &h)
    {
        if (h.size() != _img.size()) throw std::runtime_error("ImageBuffer::upload: size mismatch");
        _img.upload(h.data());
    }
    void writeToFile(fs::path filename) const
    {
        const std::vector<uchar4> h = download();
        if (!fvc_cpp::write_png(filename, reinterpret_cast<const uint8_t *>(h.data()), _res.x, _res.y))
            throw std::runtime_error("cannot write " + filename.string());
    }
    /* PSNR over the RGB channels of the two 8-bit images (src/util/image_buffer.cu:184-199) */
    float computePSNR(ImageBuffer &ref) const
    {
        if (ref._res.x != _res.x || ref._res.y != _res.y) throw std::runtime_error("PSNR computation only supported for same size images");
        const std::vector<uchar4> a = download(), b = ref.download();
        double se = 0.0;
        for (size_t i = 0; i < a.size(); ++i) {
            const double dr = (a[i].x - b[i].x) / 255.0, dg = (a[i].y - b[i].y) / 255.0, db = (a[i].z - b[i].z) / 255.0;
            se += (dr * dr + dg * dg + db * db) / 3.0;
        }
        const double mse = se / std::max<size_t>(1, a.size());
        return mse <= 0.0 ? INFINITY : (float)(-10.0 * std::log10(mse));
    }
    float computePSNR(ImageBuffer &ref, bool write_diff_image, fs::path diff_img_filename) const
    {
        const float p = computePSNR(ref);
        if (write_diff_image) {
            std::vector<uchar4> a = download();
            const std::vector<uchar4> b = ref.download();
            for (size_t i = 0; i < a.size(); ++i) {
                const int d = std::max({std::abs(a[i].x - b[i].x), std::abs(a[i].y - b[i].y), std::abs(a[i].z - b[i].z)});
                a[i] = make_uchar4((unsigned char)d, (unsigned char)d, (unsigned char)d, 255);
            }
            fvc_cpp::write_png(diff_img_filename, reinterpret_cast<const uint8_t *>(a.data()), _res.x, _res.y);
        }
        return p;
    }

private:
    int2 _res{0, 0};
    CudaBuffer<uchar4> _img;
    CudaBuffer<float4> _rgbt;
};

/* DebugBuffer<T>, include/util/image_buffer.h: per-pixel scalar buffer. */
template <typename T>
class DebugBuffer {
public:
    explicit DebugBuffer(int2 r) : _res(r), _buf((size_t)r.x * r.y) { set(T(0)); }
    void set(T v)
    {
        std::vector<T> h(_buf.size(), v);
        _buf.upload(h.data());
    }
    int2 resolution() const { return _res; }
    T *data() { return _buf.data(); }
    /* one-channel PNG through a value -> byte converter (src/util/debug_buffer.cu:69-89, PNG only) */
    void writeToFile(fs::path filename, std::function<unsigned char(T)> converter) const
    {
        std::vector<T> h;
        _buf.download(h);
        std::vector<uint8_t> g(h.size());
        std::transform(h.begin(), h.end(), g.begin(), converter);
        if (filename.extension() != ".png") throw std::runtime_error("Image file extension not supported!");
        if (!fvc_cpp::write_png(filename, g.data(), _res.x, _res.y, 1)) throw std::runtime_error("cannot write " + filename.string());
    }
    std::vector<T> download() const
    {
        std::vector<T> h;
        _buf.download(h);
        return h;
    }

private:
    int2 _res;
    CudaBuffer<T> _buf;
};

/* DebugData, include/renderer.h:72-75: the cache renderers add the
 * contribution weights of resampled samples to buffers[0] and of cache
 * samples to buffers[1] (src/cache_performance_renderer.cu:889-898). */
struct DebugData {
    std::vector<DebugBuffer<float> *> buffers;
};

/* createMinMaxConverter (include/util/bmpwriter.h:22-27) */
template <typename T>
std::function<unsigned char(T)> createMinMaxConverter(T min_val, T max_val)
{
    return [min_val, max_val](T x) -> unsigned char {
        return (unsigned char)((float)(std::min(std::max(x, min_val), max_val) - min_val) / (max_val - min_val) * 255.0f);
    };
}

/* CudaTimer (include/util/cuda_timer.h), reduced to what the renderers here
 * measure: wall time of each synchronous render and the summed CUDA-event
 * time of the resample network kernel. */
class CudaTimer {
public:
    void reset() { _ms.clear(); }
    void add(const std::string &name, float ms) { _ms[name] += ms; }
    std::map<std::string, float> getTimings(int n_iterations) const
    {
        std::map<std::string, float> r;
        for (const auto &kv : _ms) r[kv.first] = kv.second / std::max(1, n_iterations);
        return r;
    }
    void print() const
    {
        for (const auto &kv : _ms) std::cout << kv.first << ": " << kv.second << " ms" << std::endl;
    }

private:
    std::map<std::string, float> _ms;
};

/* ------------------------------------------------------------------------ */
/* renderers                                                                 */
/* ------------------------------------------------------------------------ */

struct Renderer {
    Renderer(SceneInfo scene_info, CudaBuffer<uint8_t> &occupancy_grid, NerfNetwork<half> &nerf_network, int kind)
        : _scene_info(scene_info), _occupancy_grid(occupancy_grid), _nerf_network(nerf_network)
    {
        fvc_cpp::check(fvc_renderer_create(nerf_network._model, kind, &_handle));
        fvc_cpp::check(fvc_renderer_set_kernel_timing(_handle, 1));
    }
    Renderer(const Renderer &) = delete;
    Renderer &operator=(const Renderer &) = delete;
    virtual ~Renderer() { fvc_renderer_destroy(_handle); }

    virtual void render(RaymarchInfo rm_info, RenderBuffer &render_buffer, DebugData *debug_data = nullptr) = 0;
    virtual void resizeRenderbuffers(int2 resolution) = 0;

    SceneInfo _scene_info;
    CudaBuffer<uint8_t> &_occupancy_grid;
    NerfNetwork<half> &_nerf_network;
    CudaTimer _timer;
    fvc_renderer *_handle = nullptr;

protected:
    /* one synchronous render into the buffer; returns the frame statistics */
    fvc_render_stats_t render_into(const RaymarchInfo &rm_info, RenderBuffer &buf, DebugData *debug = nullptr)
    {
        const int2 r = buf.resolution();
        if (r.x != rm_info.cam_info.resolution.x || r.y != rm_info.cam_info.resolution.y)
            throw std::runtime_error("render buffer resolution does not match the camera");
        fvc_render_outputs out{};
        out.image_rgba8 = reinterpret_cast<uint8_t *>(buf.image_device());
        out.results = reinterpret_cast<fvc_ray_result *>(buf.results_device());
        if (debug && debug->buffers.size() >= 2) {
            out.contrib_resample = debug->buffers[0]->data();
            out.contrib_cache = debug->buffers[1]->data();
        }
        const auto t0 = std::chrono::steady_clock::now();
        fvc_cpp::check(fvc_render_device(_handle, fvc_cpp::abi(rm_info), &out));
        fvc_cpp::check(fvc_renderer_synchronize(_handle));
        const float ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        fvc_render_stats_t st{};
        fvc_cpp::check(fvc_render_stats(_handle, &st));
        _timer.add("render", ms);
        _timer.add("inference resample", st.timed_kernel_ms);
        return st;
    }
};

/* PerformanceRenderer, include/performance_renderer.h:19-64. */
struct PerformanceRenderer : public Renderer {
    PerformanceRenderer(SceneInfo s, CudaBuffer<uint8_t> &g, NerfNetwork<half> &n) : Renderer(s, g, n, FVC_RENDERER_PERFORMANCE) {}
    void render(RaymarchInfo rm_info, RenderBuffer &b, DebugData * = nullptr) override
    {
        _render_stats.samples_ppx = (float)render_into(rm_info, b).samples_ppx;
    }
    void resizeRenderbuffers(int2 r) override { fvc_cpp::check(fvc_renderer_resize(_handle, r.x, r.y)); }

    static constexpr int MAX_SUBITER = 1000;
    static constexpr int TARGET_BATCH_SIZE = 1 << 21;
    struct RenderStats {
        float samples_ppx;
    } _render_stats{0.0f};
};

/* BasicRenderer, include/basic_renderer.h:10-40 (the same kernels here). */
struct BasicRenderer : public Renderer {
    BasicRenderer(SceneInfo s, CudaBuffer<uint8_t> &g, NerfNetwork<half> &n) : Renderer(s, g, n, FVC_RENDERER_BASIC) {}
    void render(RaymarchInfo rm_info, RenderBuffer &b, DebugData * = nullptr) override
    {
        _render_stats.samples_ppx = (float)render_into(rm_info, b).samples_ppx;
    }
    void resizeRenderbuffers(int2 r) override { fvc_cpp::check(fvc_renderer_resize(_handle, r.x, r.y)); }
    struct RenderStats {
        float samples_ppx;
    } _render_stats{0.0f};
};

/* Cache, include/cache.h:12-74 (storage lives in libfvc.so). */
struct Cache {
    Cache() { fvc_cpp::check(fvc_cache_create(&_handle)); }
    Cache(const Cache &) = delete;
    Cache &operator=(const Cache &) = delete;
    ~Cache() { fvc_cache_destroy(_handle); }
    fvc_cache *_handle = nullptr;
};

enum DensityInterpolVariant { Density = 0, Alpha = 1, Intermediates = 2, DensityIntermediates = 3, AlphaIntermediates = 4 };
enum InterpolFunction { Linear = 0, Smoothstep = 1, Smootherstep = 2, Nearest = 3 };

/* CacheSettings, include/cache_renderer.h:24-32. */
struct CacheSettings {
    DensityInterpolVariant interpol_variant;
    InterpolFunction interpol_function;
    bool use_hw_interpol;
    bool reweight_intermediates;
    bool disable_reweighting_first_intermediate;
    bool use_inter_brick_interpolation;
};

/* CacheRenderer, include/cache_renderer.h:34-109. */
struct CacheRenderer : public Renderer {
    CacheRenderer(SceneInfo s, CudaBuffer<uint8_t> &g, NerfNetwork<half> &n, Cache *cache, Cache *next_cache,
                  int kind = FVC_RENDERER_CACHE_PERFORMANCE)
        : Renderer(s, g, n, kind), _cache(cache), _cache_next(next_cache)
    {
        fvc_cpp::check(fvc_renderer_set_caches(_handle, cache->_handle, next_cache->_handle));
        setCacheSettings(default_cache_settings);
    }

    void resizeCache(int2 resolution, StepsizeInfo stepsize_info)
    {
        fvc_cpp::check(fvc_cache_resize(_handle, resolution.x, resolution.y, fvc_cpp::abi(stepsize_info)));
    }
    /* the per-ray fill of the next cache (src/cache_renderer.cu:848-928): sizes
     * the cache and the render buffers to the view as the reference does; the
     * debug buffer is not written */
    void initCache(RaymarchInfo rm_info, RenderBuffer &)
    {
        resizeCache(rm_info.cam_info.resolution, rm_info.stepsize_info);
        fvc_cpp::check(fvc_renderer_resize(_handle, rm_info.cam_info.resolution.x, rm_info.cam_info.resolution.y));
        fvc_cpp::check(fvc_cache_build_per_ray(_handle, fvc_cpp::abi(rm_info)));
        fvc_cache_stats_t st{};
        fvc_cpp::check(fvc_cache_stats(_handle, &st));
        const float n_rays = (float)std::max(1, rm_info.cam_info.resolution.x * rm_info.cam_info.resolution.y);
        _init_stats.samples_ppx = (float)st.n_samples / n_rays; /* :920 */
        _init_stats.n_bricks_set = st.n_bricks_set;
        _init_stats.n_bricks_reserved = st.n_bricks_reserved;
    }
    /* fills the next cache (src/cache_renderer.cu:931-1051); the debug buffer is not written */
    void initCacheBlockwise(RaymarchInfo rm_info, RenderBuffer &)
    {
        fvc_cpp::check(fvc_cache_build(_handle, fvc_cpp::abi(rm_info)));
        fvc_cache_stats_t st{};
        fvc_cpp::check(fvc_cache_stats(_handle, &st));
        _init_stats.samples_ppx = 0.0f;  /* as src/cache_renderer.cu:1048 */
        _init_stats.n_bricks_set = st.n_bricks_set;
        _init_stats.n_bricks_reserved = st.n_bricks_reserved;
    }
    void swapCache()
    {
        fvc_cpp::check(fvc_cache_swap(_handle));
        std::swap(_cache, _cache_next);
    }
    void setCacheSettings(CacheSettings s)
    {
        fvc_cache_settings c{(int)s.interpol_variant, (int)s.interpol_function, s.use_hw_interpol, s.reweight_intermediates,
                             s.disable_reweighting_first_intermediate, s.use_inter_brick_interpolation};
        fvc_cpp::check(fvc_renderer_set_cache_settings(_handle, &c));
        cache_settings = s;
    }

    static constexpr int MAX_SUBITER = 1000;
    static constexpr int TARGET_BATCH_SIZE = 1 << 21;
    static constexpr CacheSettings default_cache_settings{Density, Linear, true, true, true, true};
    CacheSettings cache_settings = default_cache_settings;
    Cache *_cache;
    Cache *_cache_next;

    struct InitStats {
        float samples_ppx;
        int n_bricks_set;
        int n_bricks_reserved;
    } _init_stats{0.0f, 0, 0};
};

/* CachePerformanceRenderer, include/cache_performance_renderer.h:21-131. */
struct CachePerformanceRenderer : public CacheRenderer {
    enum RenderMode { BOTH = 0, ONLY_CACHE = 1, ONLY_RESAMPLED = 2 };

    CachePerformanceRenderer(SceneInfo s, CudaBuffer<uint8_t> &g, NerfNetwork<half> &n, Cache *cache, Cache *next_cache)
        : CacheRenderer(s, g, n, cache, next_cache) {}

    void render(RaymarchInfo rm_info, RenderBuffer &b, DebugData *debug_data = nullptr) override
    {
        fvc_cpp::check(fvc_renderer_set_render_mode(_handle, (int)_render_mode));
        const fvc_render_stats_t st = render_into(rm_info, b, debug_data);
        const float n_rays = (float)std::max(1, rm_info.cam_info.resolution.x * rm_info.cam_info.resolution.y);
        _render_stats.samples_ppx = (float)st.samples_ppx;
        _render_stats.resample_samples_evaluated = (float)st.n_resamples / n_rays;
        _render_stats.cache_samples_evaluated = (float)st.n_cache_hits / n_rays;
        _render_stats.n_resamples = (uint64_t)st.n_resamples;
        _render_stats.n_cache_hits = (uint64_t)st.n_cache_hits;
    }
    void resizeRenderbuffers(int2 r) override { fvc_cpp::check(fvc_renderer_resize(_handle, r.x, r.y)); }

    RenderMode _render_mode = BOTH;
    struct RenderStats {
        float samples_ppx = 0;
        float resample_samples_evaluated = 0.f;
        float cache_samples_evaluated = 0.f;
        uint64_t n_resamples = 0;
        uint64_t n_cache_hits = 0;
    } _render_stats;
};

/* CacheBasicRenderer, include/cache_basic_renderer.h:10-40: the cached render
 * with the basic renderer's per-sample semantics (the cache decides by the
 * voxel's isset; every CacheSettings field applies; a cache sample composites
 * with its looked-up density). */
struct CacheBasicRenderer : public CacheRenderer {
    CacheBasicRenderer(SceneInfo s, CudaBuffer<uint8_t> &g, NerfNetwork<half> &n, Cache *cache, Cache *next_cache)
        : CacheRenderer(s, g, n, cache, next_cache, FVC_RENDERER_CACHE_BASIC) {}

    void render(RaymarchInfo rm_info, RenderBuffer &b, DebugData * = nullptr) override
    {
        const int2 r = b.resolution();
        if (r.x != rm_info.cam_info.resolution.x || r.y != rm_info.cam_info.resolution.y)
            throw std::runtime_error("render buffer resolution does not match the camera");
        if (_counts.size() != (size_t)r.x * r.y) _counts.resize((size_t)r.x * r.y);
        fvc_render_outputs out{};
        out.image_rgba8 = reinterpret_cast<uint8_t *>(b.image_device());
        out.results = reinterpret_cast<fvc_ray_result *>(b.results_device());
        out.ray_counts = reinterpret_cast<int32_t *>(_counts.data());
        fvc_cpp::check(fvc_render_device(_handle, fvc_cpp::abi(rm_info), &out));
        fvc_cpp::check(fvc_renderer_synchronize(_handle));
        fvc_render_stats_t st{};
        fvc_cpp::check(fvc_render_stats(_handle, &st));
        _render_stats.total_n_evaluated_samples_resample = (int)st.n_resamples;
        _render_stats.total_n_evaluated_samples_cache = (int)st.n_cache_hits;
    }
    void resizeRenderbuffers(int2 r) override { fvc_cpp::check(fvc_renderer_resize(_handle, r.x, r.y)); }

    /* writeImageBuffer_cacheBasic_postRender_kernel (src/cache_basic_renderer.cu:
     * 308-330): white where a cache sample contributed, and the contributing
     * sample totals, from the last render's per-pixel counts */
    void postRender(RaymarchInfo rm_info, RenderBuffer &additional_image_buffer)
    {
        const size_t n = (size_t)rm_info.cam_info.resolution.x * rm_info.cam_info.resolution.y;
        if (_counts.size() != n) throw std::runtime_error("postRender: no render at this resolution");
        std::vector<int4> counts;
        _counts.download(counts);
        std::vector<uchar4> img(n);
        long long res = 0, cache = 0;
        for (size_t i = 0; i < n; ++i) {
            res += counts[i].x;
            cache += counts[i].y;
            const unsigned char v = counts[i].y > 0 ? 255 : 0;
            img[i] = make_uchar4(v, v, v, 255);
        }
        fvc_cpp::check_cuda(cudaMemcpy(additional_image_buffer.image_device(), img.data(), n * sizeof(uchar4), cudaMemcpyHostToDevice),
                            "postRender image");
        _render_stats.total_n_contributing_samples_resample = (int)res;
        _render_stats.total_n_contributing_samples_cache = (int)cache;
    }

    struct RenderStats {
        int total_n_evaluated_samples_resample = 0;
        int total_n_contributing_samples_resample = 0;
        int total_n_evaluated_samples_cache = 0;
        int total_n_contributing_samples_cache = 0;
    } _render_stats;
    CudaBuffer<int4> _counts; /* per pixel: resample, cache, dropped samples, steps */
};
