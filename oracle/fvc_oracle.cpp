/*
 * fvc_oracle.cpp - CPU oracle for the frustum-volume-caching renderer.
 *
 * TEST INFRASTRUCTURE ONLY.  The product never links, loads or calls this
 * file; tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it
 * as the checker.
 *
 * A scalar restatement of the reference's hot path:
 *   - marcher index math in float32, operation for operation in the order the
 *     reference writes it (include/raymarch_common.h, include/common.h),
 *     compiled with -ffp-contract=off so it is bit-identical to the device;
 *   - network (hash grid + MLPs) and compositing in float64;
 *   - cache build and cached render as single-pass loops equivalent to the
 *     reference's sub-iterated kernels, with deterministic brick slots
 *     (iteration-major, then tile index) in place of the reference's
 *     atomicAdd order.
 * Each function cites the reference lines it restates.  The hash grid and
 * MLP restate the published Instant-NGP method (tiny-cuda-nn is not in the
 * reference tree); parity against tiny-cuda-nn itself is unpinned.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <mutex>
#include <vector>

#include "../frustumvolumecaching_gb300/csrc/fvc_detmath.h"
#include "../frustumvolumecaching_gb300/csrc/fvc_sampling.h"

namespace {

struct V3 { float x, y, z; };
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }

/* ---------------- parameter blocks passed from Python (ctypes) ----------- */
extern "C" {
struct OrcScene {
    int grid_nlvl; int normalized; int contraction; int is_open_gl;
    float aabb_from[3], aabb_to[3], c_from[3], c_to[3];
    float alpha_thre;
};
struct OrcSteps {  /* StepsizeInfo, include/common.h:93-107, plus L_lo */
    float cone_angle, log1p_c, stepsize, near_, near_i, far_;
    float dt_min, dt_max, t_min, t_max, i_min, i_max;
    float log1p_c_lo; int use_libm;
};
struct OrcCam {    /* CameraInfo, include/common.h:166-180, plus RaymarchInfo's sampling fields */
    int W, H; int is_open_gl; float fx, fy, px, py;
    float c2w[12]; float w2c[12];
    int nd;                /* 1: RaymarchInfo::deterministic = false */
    int motion_blur;       /* RaymarchInfo::motion_blur */
    int sample_index;      /* RaymarchInfo::sample_index */
    float aperature, focus_z;
    float nc2w[12];        /* next_cam_info.cam2world (motion blur) */
};
struct OrcNet {
    int n_levels, F;
    float scale[32]; uint32_t res[32], size[32], offset[32], dense[32];
    const uint16_t *table;   /* fp16 bits */
    int width, enc_w, enc_w_pad, base_out_pad;
    const uint16_t *base_w;  /* [width x enc_w_pad] then [base_out_pad x width] */
    int head_layers;         /* number of weight matrices in the head (3 = 2 hidden) */
    int head_in, head_in_pad, n_latents, latent_offset;
    const uint16_t *head_w;  /* [width x head_in_pad], [width x width]*, [16 x width] */
    int mimic_fp16;          /* round layer outputs to fp16 like the reference */
    int view_dependent;      /* split head (mlp_first_head, include/nerf_network.h:120-158) */
    const uint16_t *first_w; /* the first head: [width x 32], [16 x width] */
    int freq_deg;            /* the head's positional frequency encoding degree (0 or 4) */
};
}

/* ---------------- fp16 helpers ---------------- */
inline double h2d(uint16_t h)
{
    const int s = h >> 15, e = (h >> 10) & 31, m = h & 1023;
    double v;
    if (e == 0) v = std::ldexp((double)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((double)(m | 1024), e - 25);
    return s ? -v : v;
}
inline double round_h(double x) { return (double)(_Float16)(float)x; }
inline uint16_t d2h_bits(double x) { _Float16 h = (_Float16)(float)x; uint16_t b; std::memcpy(&b, &h, 2); return b; }

/* ---------------- step grid: StepsizeInfo, include/common.h:133-163 ------ */
inline float t_from_step(const OrcSteps &s, float step)
{
    if (s.cone_angle <= 0.0f) return step * s.dt_min;
    if (step >= s.i_max) return s.t_max + (step - s.i_max) * s.dt_max;
    if (step < s.i_min) return step * s.dt_min;
    if (s.use_libm) return s.t_min * powf(1.f + s.cone_angle, step - s.i_min);
    return s.t_min * fvc_pow_1pc(step - s.i_min, s.log1p_c, s.log1p_c_lo);
}
inline float step_from_t(const OrcSteps &s, float t)
{
    if (s.cone_angle <= 0.0f) return t / s.dt_min;
    if (t >= s.t_max) return (t - s.t_max) / s.dt_max + s.i_max;
    if (t < s.t_min) return t / s.dt_min;
    const float lg = s.use_libm ? logf(t / s.t_min) : fvc_logf(t / s.t_min);
    return lg / s.log1p_c + s.i_min;
}
/* calculate_stepsize + clamp, include/raymarch_common.h:274-284,
 * include/util/helper_math.h:1169-1172 */
inline float calc_step(const OrcSteps &s, float t)
{
    return fmaxf(s.dt_min, fminf(t * s.cone_angle, s.dt_max));
}
/* valid_t_from_t, include/raymarch_common.h:286-296 */
inline float valid_t_from_t(const OrcSteps &s, float t)
{
    return t_from_step(s, roundf(step_from_t(s, fmaxf(t, s.near_)) - s.near_i) + s.near_i);
}

/* ---------------- vector helpers in the reference's order --------------- */
inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot4(float ax, float ay, float az, float aw, const float *m)
{
    return ax * m[0] + ay * m[1] + az * m[2] + aw * m[3];
}

struct Ray { V3 o, d; };

/* generateRayDir + generateRay, include/raymarch_common.h:190-251, with the
 * initRayPayloads screen point (src/renderer.cu:105-108): the pixel centre,
 * or with deterministic = false the pixel plus ld_random_pixel_offset, the
 * camera slerped toward next_cam_info for motion blur (ld_random_val seeded
 * by the pixel index) and the thin-lens offset for depth of field. */
inline Ray generate_ray(const OrcCam &c, int px, int py)
{
    float ox = 0.5f, oy = 0.5f;
    if (c.nd) fvc_smp::pixel_offset((uint32_t)c.sample_index, ox, oy);
    const float sx = (float)px + ox, sy = (float)py + oy;
    float m[12];
    std::memcpy(m, c.c2w, sizeof(m));
    if (c.nd && c.motion_blur) {
        const float tm = fvc_smp::ld_val((uint32_t)c.sample_index, (uint32_t)(py * c.W + px) * 72239731u);
        fvc_smp::camera_slerp(c.c2w, c.nc2w, tm, m);
    }
    const float sgn = c.is_open_gl ? -1.f : 1.f;
    const float dx = (sx - c.px) / c.fx;
    const float dy = (sy - c.py) / c.fy * sgn;
    const float dz = sgn;
    V3 d = v3(dot4(dx, dy, dz, 0.f, m), dot4(dx, dy, dz, 0.f, m + 4), dot4(dx, dy, dz, 0.f, m + 8));
    /* normalize(): rsqrtf as the reference header evaluates it on the host
     * (nvcc host math: 1/sqrt in double, rounded once to float). */
    const float inv = (float)(1.0 / std::sqrt((double)dot3(d, d)));
    d = v3(d.x * inv, d.y * inv, d.z * inv);
    V3 o = v3(m[3], m[7], m[11]);
    if (c.nd && c.aperature != 0.0f) {
        const V3 look = v3(o.x + d.x * c.focus_z, o.y + d.y * c.focus_z, o.z + d.z * c.focus_z);
        float bx, by;
        fvc_smp::lens_offset((uint32_t)c.sample_index, sx, sy, c.W, c.H, c.aperature, bx, by);
        o.x += m[0] * bx + m[1] * by;
        o.y += m[4] * bx + m[5] * by;
        o.z += m[8] * bx + m[9] * by;
        d = v3((look.x - o.x) / c.focus_z, (look.y - o.y) / c.focus_z, (look.z - o.z) / c.focus_z);
    }
    return Ray{o, d};
}

/* the ray's first t1 (initRayPayloads_split_kernel, src/renderer.cu:119-124):
 * valid_t_from_t of the box entry, plus the first step times
 * ld_random_t_offset(sample_index, ray_id * 56924617) when not deterministic */
inline float start_t1(const OrcCam &c, const OrcSteps &st, float tn, int ray_id)
{
    const float start = valid_t_from_t(st, tn);
    const float toff = c.nd ? fvc_smp::t_offset((uint32_t)c.sample_index, (uint32_t)ray_id) : 0.0f;
    return start + calc_step(st, start) * toff;
}

/* ray_aabb_intersect, include/raymarch_common.h:482-532 */
inline bool ray_aabb(const Ray &r, const float *from, const float *to, float &tn, float &tf)
{
    float tmin = (from[0] - r.o.x) / r.d.x, tmax = (to[0] - r.o.x) / r.d.x;
    if (tmin > tmax) std::swap(tmin, tmax);
    float tymin = (from[1] - r.o.y) / r.d.y, tymax = (to[1] - r.o.y) / r.d.y;
    if (tymin > tymax) std::swap(tymin, tymax);
    if (tmin > tymax || tymin > tmax) { tn = 1e10f; tf = 1e10f; return false; }
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    float tzmin = (from[2] - r.o.z) / r.d.z, tzmax = (to[2] - r.o.z) / r.d.z;
    if (tzmin > tzmax) std::swap(tzmin, tzmax);
    if (tmin > tzmax || tzmin > tmax) { tn = 1e10f; tf = 1e10f; return false; }
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    tn = tmin; tf = tmax;
    return true;
}

/* morton3D, include/raymarch_common.h:98-110 */
inline uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) { return expand_bits(x) | (expand_bits(y) << 1) | (expand_bits(z) << 2); }
inline uint32_t compact_bits(uint32_t x)  /* morton3D_invert, :90-97 */
{
    x = x & 0x49249249u;
    x = (x | (x >> 2)) & 0xc30c30c3u;
    x = (x | (x >> 4)) & 0x0f00f00fu;
    x = (x | (x >> 8)) & 0xff0000ffu;
    x = (x | (x >> 16)) & 0x0000ffffu;
    return x;
}

constexpr int R = 128;  /* DEFAULT_GRID_RESOLUTION, include/renderer_common.h:10 */

/* grid_occupied_at<128, true>, include/raymarch_common.h:660-710 */
inline bool occupied(const OrcScene &sc, const uint8_t *bits, V3 p, int *cell_out = nullptr)
{
    V3 u = p;
    if (!sc.normalized) {
        const float s = (float)(1 << (sc.grid_nlvl - 1));
        u = v3((p.x - sc.aabb_from[0] / s) / ((sc.aabb_to[0] - sc.aabb_from[0]) / s),
               (p.y - sc.aabb_from[1] / s) / ((sc.aabb_to[1] - sc.aabb_from[1]) / s),
               (p.z - sc.aabb_from[2] / s) / ((sc.aabb_to[2] - sc.aabb_from[2]) / s));
    }
    const float mx = fmaxf(fmaxf(fabsf(u.x - 0.5f), fabsf(u.y - 0.5f)), fabsf(u.z - 0.5f));
    int e;
    frexpf(mx, &e);
    const int mip = std::max(0, e + 1);
    if (mip >= sc.grid_nlvl) { if (cell_out) *cell_out = -1; return false; }
    const float sm = scalbnf(1.0f, -mip);
    const int ix = (int)(((u.x - 0.5f) * sm + 0.5f) * (float)R);
    const int iy = (int)(((u.y - 0.5f) * sm + 0.5f) * (float)R);
    const int iz = (int)(((u.z - 0.5f) * sm + 0.5f) * (float)R);
    const int idx = (int)morton3((uint32_t)ix, (uint32_t)iy, (uint32_t)iz);
    const int bidx = idx / 8 + (R * R * R * mip) / 8;
    if (cell_out) *cell_out = bidx * 8 + idx % 8;
    return (bits[bidx] & (1 << (idx % 8))) != 0;
}

/* apply_contraction, include/raymarch_common.h:610-653 */
inline V3 contract(const OrcScene &sc, V3 p)
{
    if (sc.contraction == 1) {
        return v3((p.x - sc.aabb_from[0]) / (sc.aabb_to[0] - sc.aabb_from[0]),
                  (p.y - sc.aabb_from[1]) / (sc.aabb_to[1] - sc.aabb_from[1]),
                  (p.z - sc.aabb_from[2]) / (sc.aabb_to[2] - sc.aabb_from[2]));
    }
    if (sc.contraction == 2 || sc.contraction == 3) {
        V3 u = v3((p.x - sc.c_from[0]) / (sc.c_to[0] - sc.c_from[0]) * 2.0f - 1.0f,
                  (p.y - sc.c_from[1]) / (sc.c_to[1] - sc.c_from[1]) * 2.0f - 1.0f,
                  (p.z - sc.c_from[2]) / (sc.c_to[2] - sc.c_from[2]) * 2.0f - 1.0f);
        const float n = sc.contraction == 3 ? fmaxf(fmaxf(fabsf(u.x), fabsf(u.y)), fabsf(u.z)) : sqrtf(dot3(u, u));
        const float f = fmaxf(n, 1.0f);
        const float k = 2.0f - 1.0f / f;
        return v3(k * (u.x / f) / 4.0f + 0.5f, k * (u.y / f) / 4.0f + 0.5f, k * (u.z / f) / 4.0f + 0.5f);
    }
    return p;
}

/* transformRay, include/raymarch_common.h:253-262 */
inline Ray transform_ray(const Ray &r, const float *m)
{
    return Ray{v3(dot4(r.o.x, r.o.y, r.o.z, 1.0f, m), dot4(r.o.x, r.o.y, r.o.z, 1.0f, m + 4), dot4(r.o.x, r.o.y, r.o.z, 1.0f, m + 8)),
               v3(dot4(r.d.x, r.d.y, r.d.z, 0.0f, m), dot4(r.d.x, r.d.y, r.d.z, 0.0f, m + 4), dot4(r.d.x, r.d.y, r.d.z, 0.0f, m + 8))};
}
inline V3 at(const Ray &r, float t) { return v3(r.o.x + t * r.d.x, r.o.y + t * r.d.y, r.o.z + t * r.d.z); }

/* cam2froxel, include/raymarch_common.h:316-329 */
inline V3 cam2froxel(V3 c, const OrcCam &cam, const OrcSteps &st, float &t)
{
    const float sgn = cam.is_open_gl ? -1.f : 1.f;
    const float z = c.z * sgn;
    t = sqrtf(dot3(c, c));
    return v3(c.x / z * cam.fx + cam.px, c.y * sgn / z * cam.fy + cam.py,
              (step_from_t(st, t) - st.near_i) * (c.z < 0.0f ? -1.0f : 1.0f));
}

/* ---------------- network (float64) ---------------- */
struct NetD {
    const OrcNet *n;
    std::vector<double> table, bw0, bw1, hw[4], fw0, fw1;
};

void prepare_net(const OrcNet *n, NetD &d)
{
    d.n = n;
    size_t n_entries = (size_t)n->offset[n->n_levels - 1] + n->size[n->n_levels - 1];
    d.table.resize(n_entries * n->F);
    for (size_t i = 0; i < d.table.size(); ++i) d.table[i] = h2d(n->table[i]);
    d.bw0.resize((size_t)n->width * n->enc_w_pad);
    d.bw1.resize((size_t)n->base_out_pad * n->width);
    for (size_t i = 0; i < d.bw0.size(); ++i) d.bw0[i] = h2d(n->base_w[i]);
    for (size_t i = 0; i < d.bw1.size(); ++i) d.bw1[i] = h2d(n->base_w[d.bw0.size() + i]);
    size_t off = 0;
    for (int l = 0; l < n->head_layers; ++l) {
        const int in = l == 0 ? n->head_in_pad : n->width;
        const int out = l == n->head_layers - 1 ? 16 : n->width;
        d.hw[l].resize((size_t)in * out);
        for (size_t i = 0; i < d.hw[l].size(); ++i) d.hw[l][i] = h2d(n->head_w[off + i]);
        off += (size_t)in * out;
    }
    if (n->view_dependent) {
        d.fw0.resize((size_t)n->width * 32);
        d.fw1.resize((size_t)16 * n->width);
        for (size_t i = 0; i < d.fw0.size(); ++i) d.fw0[i] = h2d(n->first_w[i]);
        for (size_t i = 0; i < d.fw1.size(); ++i) d.fw1[i] = h2d(n->first_w[d.fw0.size() + i]);
    }
}

/* Hash-grid encoding (Instant-NGP multiresolution hash grid): the corner and
 * fraction in float32 exactly as the device computes them (p = fma(scale, x,
 * 0.5), floor, subtract), weights and sums in float64. */
void hash_encode(const NetD &d, V3 pos, double *feat)
{
    const OrcNet &n = *d.n;
    const float px[3] = {pos.x, pos.y, pos.z};
    for (int l = 0; l < n.n_levels; ++l) {
        uint32_t g[3]; double fr[3];
        for (int k = 0; k < 3; ++k) {
            const float p = fmaf(n.scale[l], px[k], 0.5f);
            const float fl = floorf(p);
            g[k] = (uint32_t)(int)fl;
            fr[k] = (double)(p - fl);
        }
        double acc[8] = {0};
        for (int c = 0; c < 8; ++c) {
            uint32_t q[3]; double w = 1.0;
            for (int k = 0; k < 3; ++k) {
                const int b = (c >> k) & 1;
                q[k] = g[k] + (uint32_t)b;
                w *= b ? fr[k] : 1.0 - fr[k];
            }
            uint32_t idx;
            if (n.dense[l]) idx = q[0] + q[1] * n.res[l] + q[2] * n.res[l] * n.res[l];
            else idx = (q[0] * 1u) ^ (q[1] * 2654435761u) ^ (q[2] * 805459861u);
            idx %= n.size[l];
            const double *e = &d.table[((size_t)n.offset[l] + idx) * n.F];
            for (int f = 0; f < n.F; ++f) acc[f] += w * e[f];
        }
        for (int f = 0; f < n.F; ++f) feat[l * n.F + f] = n.mimic_fp16 ? round_h(acc[f]) : acc[f];
    }
    for (int i = n.n_levels * n.F; i < n.enc_w_pad; ++i) feat[i] = 0.0;
}

inline void dense_layer(const double *W, int out, int in, const double *x, double *y, bool relu, bool mimic)
{
    for (int o = 0; o < out; ++o) {
        double s = 0.0;
        const double *w = W + (size_t)o * in;
        for (int i = 0; i < in; ++i) s += w[i] * x[i];
        /* ReLU maps NaN to 0, as fmaxf(x, 0) does on the GPU: a cache lookup
         * whose interpolated isset is 0 (possible with Nearest interpolation,
         * whose texel can differ from the classification's) yields 0/0
         * latents in the reference's formula */
        if (relu && !(s > 0.0)) s = 0.0;
        y[o] = mimic ? round_h(s) : s;
    }
}

void sh16(const float *d01, double *o);

/* density network: NerfNetwork::inferenceLatents, include/nerf_network.h:173-202.
 * A view-dependent network then runs its first head on [density outputs |
 * SH of the initial direction init01] (:183-197); the first head's outputs
 * take rows 1.. of out, row 0 keeps the log-density. */
void base_forward(const NetD &d, V3 pos, double *out /* base_out_pad */, const float *init01 = nullptr)
{
    const OrcNet &n = *d.n;
    double feat[64], h[128];
    hash_encode(d, pos, feat);
    dense_layer(d.bw0.data(), n.width, n.enc_w_pad, feat, h, true, n.mimic_fp16);
    dense_layer(d.bw1.data(), n.base_out_pad, n.width, h, out, false, n.mimic_fp16);
    if (n.view_dependent && init01) {
        double in[32], hf[128], o[16];
        for (int i = 0; i < 16; ++i) in[i] = out[i];
        sh16(init01, in + 16);
        if (n.mimic_fp16) for (int i = 16; i < 32; ++i) in[i] = round_h(in[i]);
        dense_layer(d.fw0.data(), n.width, 32, in, hf, true, n.mimic_fp16);
        dense_layer(d.fw1.data(), 16, n.width, hf, o, false, n.mimic_fp16);
        for (int i = 1; i < 16; ++i) out[i] = o[i - 1];
    }
}

/* SH degree 4 of unit_to_01 directions: x = 2*d01 - 1 (the constants of
 * src/my_fully_fused_mlp.cu:216-233, Sloan's real SH) */
void sh16(const float *d01, double *o)
{
    const double x = (double)(d01[0] * 2.f - 1.f), y = (double)(d01[1] * 2.f - 1.f), z = (double)(d01[2] * 2.f - 1.f);
    const double xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
    const double pi = 3.14159265358979323846;
    const double c0 = 1.0 / (2.0 * std::sqrt(pi)), c1 = std::sqrt(3.0) / (2.0 * std::sqrt(pi));
    const double c2a = std::sqrt(15.0) / (2.0 * std::sqrt(pi)), c2b = std::sqrt(5.0) / (4.0 * std::sqrt(pi));
    const double c2c = std::sqrt(15.0) / (4.0 * std::sqrt(pi)), c3a = std::sqrt(70.0) / (8.0 * std::sqrt(pi));
    const double c3b = std::sqrt(105.0) / (2.0 * std::sqrt(pi)), c3c = std::sqrt(42.0) / (8.0 * std::sqrt(pi));
    const double c3d = std::sqrt(7.0) / (4.0 * std::sqrt(pi)), c3e = std::sqrt(105.0) / (4.0 * std::sqrt(pi));
    o[0] = c0; o[1] = -c1 * y; o[2] = c1 * z; o[3] = -c1 * x;
    o[4] = c2a * xy; o[5] = -c2a * yz; o[6] = c2b * (3.0 * z2 - 1.0); o[7] = -c2a * xz;
    o[8] = c2c * (x2 - y2); o[9] = c3a * y * (-3.0 * x2 + y2); o[10] = c3b * xy * z;
    o[11] = c3c * y * (1.0 - 5.0 * z2); o[12] = c3d * z * (5.0 * z2 - 3.0); o[13] = c3c * x * (1.0 - 5.0 * z2);
    o[14] = c3e * z * (x2 - y2); o[15] = c3a * x * (-x2 + 3.0 * y2);
}

/* color head: NerfNetwork::inferenceHead, include/nerf_network.h:204-257
 * (latents, SH4 of the direction, padding with 1.0 to the padded width).  A
 * view-dependent head also reads SH(dir) - SH(init01), fp16 operands
 * subtracted in fp16 (nerf_network.h:47-52,226-240); without init01 (the
 * row's own direction) that input is zero. */
void head_forward(const NetD &d, const double *latents, const float *dir01, double *rgb_logits, const float *init01 = nullptr,
                  const V3 *pos = nullptr)
{
    const OrcNet &n = *d.n;
    double in[128], a[128], b[128];
    for (int i = 0; i < n.n_latents; ++i) in[i] = latents[i];
    sh16(dir01, in + n.n_latents);
    if (n.mimic_fp16) for (int i = n.n_latents; i < n.n_latents + 16; ++i) in[i] = round_h(in[i]);
    if (n.view_dependent) {
        double shi[16];
        if (init01) sh16(init01, shi);
        for (int i = 0; i < 16; ++i) {
            const double s0 = in[n.n_latents + i];
            in[n.n_latents + 16 + i] = !init01 ? 0.0 : n.mimic_fp16 ? round_h(s0 - round_h(shi[i])) : s0 - shi[i];
        }
    }
    if (n.freq_deg > 0) {
        /* frequency_encoding (include/nerf_network.h:55-81) of the network's input position, after the SH
         * inputs: per axis the sines of pi 2^k p, then the cosines (a phase of pi/2), k < degree */
        const int o = n.n_latents + (n.view_dependent ? 32 : 16);
        const double p3[3] = {pos ? (double)pos->x : 0.0, pos ? (double)pos->y : 0.0, pos ? (double)pos->z : 0.0};
        for (int j = 0; j < 6 * n.freq_deg; ++j) {
            const int axis = j / (2 * n.freq_deg), k = j % n.freq_deg, cosine = (j / n.freq_deg) % 2;
            const double x = M_PI * std::ldexp(p3[axis], k);
            const double v = cosine ? std::cos(x) : std::sin(x);
            in[o + j] = n.mimic_fp16 ? round_h(v) : v;
        }
    }
    for (int i = n.head_in; i < n.head_in_pad; ++i) in[i] = 1.0;
    dense_layer(d.hw[0].data(), n.width, n.head_in_pad, in, a, true, n.mimic_fp16);
    double *x = a, *y = b;
    for (int l = 1; l < n.head_layers - 1; ++l) {
        dense_layer(d.hw[l].data(), n.width, n.width, x, y, true, n.mimic_fp16);
        std::swap(x, y);
    }
    double out[16];
    dense_layer(d.hw[n.head_layers - 1].data(), 16, n.width, x, out, false, n.mimic_fp16);
    for (int i = 0; i < 3; ++i) rgb_logits[i] = out[i];
}

inline double sigmoid(double x) { return 1.0 / (1.0 + std::exp(-x)); }

/* one compositing step, accumulate_performance_kernel,
 * src/performance_renderer.cu:101-120; returns true when T < 1e-4 */
inline bool composite(double sigma, const double *logit, float dt, float alpha_thre, double *rgb, double &T)
{
    double alpha = 1.0 - std::exp(-sigma * (double)dt);
    alpha = std::min(1.0, std::max(0.0, alpha));
    if (alpha > (double)alpha_thre) {
        const double w = alpha * T;
        for (int k = 0; k < 3; ++k) rgb[k] += w * sigmoid(logit[k]);
        T *= 1.0 - alpha;
    }
    return T < 1e-4;
}

template <class F>
void parallel_rows(int n, int n_threads, F fn)
{
    if (n_threads <= 1) { for (int i = 0; i < n; ++i) fn(i); return; }
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t)
        th.emplace_back([&]() { for (int i; (i = next.fetch_add(1)) < n;) fn(i); });
    for (auto &t : th) t.join();
}

}  // namespace

/* ========================================================================== */
extern "C" {

/* StepsizeInfo::setAdditionalInfo, include/common.h:109-131 (host double). */
void orc_setup_steps(const OrcScene *sc, OrcSteps *s)
{
    s->dt_min = s->stepsize;
    s->dt_max = fmaxf(fmaxf((sc->aabb_to[0] - sc->aabb_from[0]) / R * 1.732f, (sc->aabb_to[1] - sc->aabb_from[1]) / R * 1.732f),
                      (sc->aabb_to[2] - sc->aabb_from[2]) / R * 1.732f);
    s->t_min = ((double)s->dt_min) / s->cone_angle;
    const double d_i_min = 1.0 / s->cone_angle;
    s->i_min = d_i_min;
    const double d_log1p_c = std::log(1.0 + s->cone_angle);
    s->log1p_c = d_log1p_c;
    s->log1p_c_lo = (float)(d_log1p_c - (double)s->log1p_c);
    const double d_i_max = std::log(s->dt_max / (double)s->dt_min) / d_log1p_c + d_i_min;
    s->i_max = d_i_max;
    s->t_max = s->t_min * std::pow(1.0 + s->cone_angle, d_i_max - d_i_min);
    s->near_i = step_from_t(*s, s->near_);
}

/* Morton bitfield from the export's uint8 grid (l*R^3 + x*R^2 + y*R + z):
 * occupancy_grid_to_morton_kernel + uchar_to_bitfield, src/loader.cu:20-55. */
void orc_grid_to_morton_bits(const uint8_t *grid, int nlvl, uint8_t *bits)
{
    const int vals = R * R * R;
    std::memset(bits, 0, (size_t)vals * nlvl / 8);
    for (int i = 0; i < vals * nlvl; ++i) {
        const int lvl = i / vals, j = i % vals;
        const uint32_t x = compact_bits((uint32_t)j), y = compact_bits((uint32_t)j >> 1), z = compact_bits((uint32_t)j >> 2);
        if (grid[(size_t)lvl * vals + x * R * R + y * R + z]) bits[i / 8] |= (uint8_t)(1u << (i % 8));
    }
}

/* Per-ray march trace for golden comparisons: sample_performance_kernel's
 * step loop (src/performance_renderer.cu:39-62) without compositing.
 * Writes per step the bits of t0 and the occupancy bit; returns steps. */
int orc_trace_ray(const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                  int px, int py, int max_steps, uint32_t *t0_bits, uint8_t *occ, float *init /* start_t, far, hits */)
{
    const Ray r = generate_ray(*cam, px, py);
    float tn, tf;
    const bool hits = ray_aabb(r, sc->aabb_from, sc->aabb_to, tn, tf);
    const float far_ = hits ? fminf(tf, st->far_) : st->far_;
    const float start = hits ? valid_t_from_t(*st, tn) : st->near_;
    init[0] = start; init[1] = far_; init[2] = hits ? 1.f : 0.f;
    if (!hits) return 0;
    float t1 = start + 0.0f;
    int n = 0;
    for (; n < max_steps; ++n) {
        const float t0 = t1;
        const float dt = calc_step(*st, t0);
        t1 = t0 + dt;
        const float tm = (t0 + t1) * 0.5f;
        if (tm > far_) break;
        std::memcpy(&t0_bits[n], &t0, 4);
        occ[n] = occupied(*sc, bits, at(r, tm)) ? 1 : 0;
    }
    return n;
}

/* Single-point helpers for golden vectors. */
float orc_step_from_t(const OrcSteps *st, float t) { return step_from_t(*st, t); }

/* the sampling of non-deterministic ray generation (fvc_sampling.h) */
uint32_t orc_smp_sobol(uint32_t index, uint32_t dim) { return fvc_smp::sobol(index, dim); }
float orc_smp_ld_val(uint32_t index, uint32_t seed, uint32_t dim) { return fvc_smp::ld_val(index, seed, dim); }
void orc_smp_pixel_offset(uint32_t spp, float *out) { fvc_smp::pixel_offset(spp, out[0], out[1]); }
float orc_smp_t_offset(uint32_t spp, uint32_t ray_id) { return fvc_smp::t_offset(spp, ray_id); }
void orc_smp_square_to_disk(float a, float b, float *out) { fvc_smp::square_to_disk(a, b, out[0], out[1]); }
void orc_smp_camera_slerp(const float *a, const float *b, float t, float *out)
{
    float m[12] = {0};
    fvc_smp::camera_slerp(a, b, t, m);
    std::memcpy(out, m, sizeof(m));
}
/* generate_ray of pixel (px, py) and the ray's first t1: out = origin, dir, start t1, hits */
void orc_generate_ray(const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, int px, int py, float *out)
{
    const Ray r = generate_ray(*cam, px, py);
    float tn, tf;
    const bool hits = ray_aabb(r, sc->aabb_from, sc->aabb_to, tn, tf);
    out[0] = r.o.x; out[1] = r.o.y; out[2] = r.o.z; out[3] = r.d.x; out[4] = r.d.y; out[5] = r.d.z;
    out[6] = hits ? start_t1(*cam, *st, tn, py * cam->W + px) : 0.0f;
    out[7] = hits ? 1.0f : 0.0f;
}
float orc_t_from_step(const OrcSteps *st, float s) { return t_from_step(*st, s); }
int orc_occupied(const OrcScene *sc, const uint8_t *bits, const float *p, int *cell)
{
    return occupied(*sc, bits, v3(p[0], p[1], p[2]), cell) ? 1 : 0;
}
void orc_contract(const OrcScene *sc, const float *p, float *out)
{
    V3 c = contract(*sc, v3(p[0], p[1], p[2]));
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}
float orc_logf(float x) { return fvc_logf(x); }
float orc_expf(float x) { return fvc_expf(x); }

/* Network evaluation at given inputs (float64): out[4n] = rgb logits, log-density. */
void orc_inference(const OrcNet *net, const float *pos, const float *dir01, int n, double *out, int n_threads)
{
    NetD d; prepare_net(net, d);
    parallel_rows(n, n_threads, [&](int i) {
        double bo[64];
        const V3 p = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        base_forward(d, p, bo, dir01 + 3 * i);
        double lg[3];
        head_forward(d, bo + net->latent_offset, dir01 + 3 * i, lg, nullptr, &p);
        out[4 * i + 0] = lg[0]; out[4 * i + 1] = lg[1]; out[4 * i + 2] = lg[2]; out[4 * i + 3] = bo[0];
    });
}
/* The density network's outputs at given inputs (float64, base_out_pad per
 * row; row 0 the log-density): what NerfNetwork::inferenceLatents writes for
 * a model without a first head (include/nerf_network.h:173-202). */
void orc_base_outputs(const OrcNet *net, const float *pos, const float *dir01, int n, double *out, int n_threads)
{
    NetD d; prepare_net(net, d);
    parallel_rows(n, n_threads, [&](int i) {
        double bo[64];
        base_forward(d, v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), bo, dir01 + 3 * i);
        for (int j = 0; j < net->base_out_pad; ++j) out[(size_t)i * net->base_out_pad + j] = bo[j];
    });
}
void orc_hash_encode(const OrcNet *net, const float *pos, int n, double *feat_out)
{
    NetD d; prepare_net(net, d);
    for (int i = 0; i < n; ++i) hash_encode(d, v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), feat_out + (size_t)i * net->enc_w_pad);
}

/* Plain render: PerformanceRenderer::render (src/performance_renderer.cu:214-286)
 * as a single pass per ray (sub-iterations only batch the same sample sequence).
 * results[4*W*H] = rgb, transmittance; n_samples[W*H]; n_steps[W*H]. */
int orc_render_plain(const OrcNet *net, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                     int row0, int row1, float *results, int32_t *n_samples, int32_t *n_steps, int n_threads)
{
    NetD d; prepare_net(net, d);
    const int W = cam->W;
    parallel_rows(row1 - row0, n_threads, [&](int rr) {
        const int y = row0 + rr;
        for (int x = 0; x < W; ++x) {
            const size_t id = (size_t)y * W + x;
            const Ray r = generate_ray(*cam, x, y);
            float tn, tf;
            const bool hits = ray_aabb(r, sc->aabb_from, sc->aabb_to, tn, tf);
            double rgb[3] = {0, 0, 0}, T = 1.0;
            int ns = 0, nst = 0;
            if (hits) {
                const float far_ = fminf(tf, st->far_);
                float t1 = start_t1(*cam, *st, tn, (int)id);
                const float d01[3] = {(r.d.x + 1.0f) / 2.0f, (r.d.y + 1.0f) / 2.0f, (r.d.z + 1.0f) / 2.0f};
                for (;;) {
                    const float t0 = t1;
                    const float dt = calc_step(*st, t0);
                    t1 = t0 + dt;
                    const float tm = (t0 + t1) * 0.5f;
                    ++nst;
                    if (tm > far_) break;
                    const V3 wp = at(r, tm);
                    if (!occupied(*sc, bits, wp)) continue;
                    double bo[64], lg[3];
                    const V3 cp = contract(*sc, wp);
                    base_forward(d, cp, bo, d01);
                    head_forward(d, bo + net->latent_offset, d01, lg, nullptr, &cp);
                    ++ns;
                    if (composite(std::exp(bo[0]), lg, dt, sc->alpha_thre, rgb, T)) break;
                }
            }
            results[4 * id + 0] = (float)rgb[0]; results[4 * id + 1] = (float)rgb[1];
            results[4 * id + 2] = (float)rgb[2]; results[4 * id + 3] = (float)T;
            if (n_samples) n_samples[id] = ns;
            if (n_steps) n_steps[id] = nst;
        }
    });
    return 0;
}

/* ---------------- frustum volume cache ---------------- */
struct OrcCacheDims {
    int fW, fH, fD;           /* frustum dims */
    int bX, bY, bZ;           /* brick dims = ceil(frustum / 8) */
    int dX, dY, dZ;           /* data bricks per dim (128, 128, z) */
};

/* CacheRenderer::resizeCache + Cache::resize (src/cache_renderer.cu:832-846,
 * src/cache.cu:44-84). */
void orc_cache_dims(const OrcScene *sc, const OrcSteps *st, int W, int H, OrcCacheDims *cd)
{
    const int n_rays = W * H;
    const int est_samples = n_rays * 32;               /* INIT_ESTIMATED_N_SAMPLES_PER_RAY */
    const int est_per_brick = (int)(0.5f * powf(8.0f, 3.0f)); /* INIT_ESTIMATED_BRICK_SPARSITY * 8^3 */
    const int est_bricks = est_samples / est_per_brick;
    const float dx = sc->aabb_to[0] - sc->aabb_from[0], dy = sc->aabb_to[1] - sc->aabb_from[1], dz = sc->aabb_to[2] - sc->aabb_from[2];
    const float diag = sqrtf(dx * dx + dy * dy + dz * dz);  /* max_step_in_scene, include/raymarch_common.h:298-303 */
    const int max_n_steps = (int)ceilf(step_from_t(*st, diag + st->near_));
    const int depth = (max_n_steps + 3) / 4 * 4;
    cd->fW = W; cd->fH = H; cd->fD = depth;
    cd->bX = (W + 7) / 8; cd->bY = (H + 7) / 8; cd->bZ = (depth + 7) / 8;
    cd->dX = 1024 / 8; cd->dY = 1024 / 8;
    cd->dZ = (est_bricks + cd->dX * cd->dY - 1) / (cd->dX * cd->dY);
}

struct OrcCache {
    OrcCacheDims dims;
    int32_t *packed_index;   /* [bZ][bY][bX] (x fastest), pack3D(slot) or -1 */
    float *known_ranges;     /* [H][W] */
    float *vox_density;      /* [slots][512] */
    float *vox_isset;        /* [slots][512] */
    uint16_t *vox_latents;   /* [slots][512][8] fp16 */
    /* stats out */
    int n_bricks_set, n_demanded, n_iterations;
    long long n_samples;
    int32_t *slot_of_brick_order; /* optional: [capacity] tile index per slot (may be NULL) */
    /* CacheSettings (include/cache_renderer.h:24-32): interpol_variant steers
     * what a build stores and how a lookup forms the head input;
     * interpol_function the trilinear weights of a lookup */
    int variant, interp;
    /* the basic cache renderer's semantics (CacheBasicRenderer) and the
     * CacheSettings flags only it reads */
    int basic, reweight, keep_first, inter_brick;
};

/* applyInterpolationFunction, include/raymarch_common.h:393-402, with the
 * smoothstep / smootherstep polynomials of
 * include/util/helper_math_extension.h:146-181; float as the reference */
inline float interp_fn(float t, int fn)
{
    if (fn == 1) return (t * t) * (3.0f - 2.0f * t);
    if (fn == 2) return ((t * t) * t) * (t * (6.0f * t - 15.0f) + 10.0f);
    if (fn == 3) return nearbyintf(t);
    return t;
}

inline int pack3(int x, int y, int z) { return (x << 20) | (y << 10) | z; }

/* Cache build: CacheRenderer::initCacheBlockwise and its kernels
 * (src/cache_renderer.cu:18-569, 931-1051) with brick slots assigned in
 * (iteration, tile index) order.  The cache camera's rays are generated
 * per 8x8 tile including pixels beyond the image (as the reference does). */
int orc_cache_build(const OrcNet *net, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                    OrcCache *cc, int n_threads)
{
    NetD d; prepare_net(net, d);
    const OrcCacheDims &cd = cc->dims;
    const int nT = cd.bX * cd.bY;
    const int capacity = cd.dX * cd.dY * cd.dZ;
    struct RayS { Ray r; float far_; bool alive; double T; };
    std::vector<RayS> rays((size_t)nT * 64);
    std::vector<int> block_step(nT), alive_tile(nT), n_bricks(nT, 0);
    std::fill(cc->packed_index, cc->packed_index + (size_t)cd.bX * cd.bY * cd.bZ, -1);
    /* initPayloads_cache_init_kernel, :18-81 */
    for (int t = 0; t < nT; ++t) {
        const int tx = t % cd.bX, ty = t / cd.bX;
        int n_alive = 0, min_start = 1 << 30;
        for (int k = 0; k < 64; ++k) {
            const int px = tx * 8 + (k % 8), py = ty * 8 + (k / 8);
            RayS &rs = rays[(size_t)t * 64 + k];
            rs.r = generate_ray(*cam, px, py);
            float tn, tf;
            const bool hits = ray_aabb(rs.r, sc->aabb_from, sc->aabb_to, tn, tf);
            n_alive += hits;
            const int start_step = std::max(0, (int)(step_from_t(*st, hits ? tn : st->near_) - st->near_i));
            min_start = std::min(min_start, start_step);
            rs.far_ = hits ? fminf(tf, st->far_) : st->far_;
            rs.alive = hits; rs.T = 1.0;
        }
        block_step[t] = min_start / 8;
        alive_tile[t] = n_alive > 0;
    }
    int counter = 0;
    long long n_samples = 0;
    int iter = 0;
    struct TileWork { int n_steps; int need; std::vector<uint8_t> mask; std::vector<double> sig, alpha, lat; };
    std::vector<TileWork> work(nT);
    for (; iter < 1000; ++iter) {
        std::vector<int> alive_list;
        for (int t = 0; t < nT; ++t) if (alive_tile[t]) alive_list.push_back(t);
        if (alive_list.empty()) break;
        /* sample_cache_init_first_kernel (:83-190): find the next depth brick
         * holding an occupied sample, then the network and the density-only
         * compositing of accumulateNew_cache_init_second_kernel (:289-528). */
        parallel_rows((int)alive_list.size(), n_threads, [&](int ai) {
            const int t = alive_list[ai];
            TileWork &w = work[t];
            w.n_steps = 0; w.need = 0;
            w.mask.assign(64, 0);
            RayS *rs = &rays[(size_t)t * 64];
            int total = 0;
            for (;;) {
                int n_alive = 0;
                for (int k = 0; k < 64; ++k) n_alive += rs[k].alive;
                if (n_alive <= 0) break;
                /* bricks beyond the frustum depth (camera outside the scene
                 * box) have no storage: the tile stops there */
                if (block_step[t] >= cd.bZ) { for (int k = 0; k < 64; ++k) rs[k].alive = false; total = 0; break; }
                const float t1s = t_from_step(*st, (float)(block_step[t] * 8) + st->near_i);
                total = 0;
                for (int k = 0; k < 64; ++k) {
                    float t1 = t1s; uint8_t m = 0;
                    for (int s = 0; s < 8; ++s) {
                        const float t0 = t1; const float dt = calc_step(*st, t0); t1 = t0 + dt;
                        const float tm = (t0 + t1) * 0.5f;
                        if (tm > rs[k].far_) rs[k].alive = false;
                        else if (occupied(*sc, bits, at(rs[k].r, tm))) { m |= (uint8_t)(1u << s); ++total; }
                    }
                    w.mask[k] = m;
                }
                if (total > 0) break;
                block_step[t]++;
            }
            int n_alive = 0;
            for (int k = 0; k < 64; ++k) n_alive += rs[k].alive;
            alive_tile[t] = n_alive > 0;
            w.n_steps = total;
            if (total == 0 || !alive_tile[t]) return;
            w.sig.assign(64 * 8, 0.0); w.alpha.assign(64 * 8, 0.0); w.lat.assign(64 * 8 * 8, 0.0);
            const float t1s = t_from_step(*st, (float)(block_step[t] * 8) + st->near_i);
            int visible = 0;
            for (int k = 0; k < 64; ++k) {
                float t1 = t1s;
                double T = rs[k].T;
                for (int s = 0; s < 8; ++s) {
                    const float t0 = t1; const float dt = calc_step(*st, t0); t1 = t0 + dt;
                    const float tm = (t0 + t1) * 0.5f;
                    if (tm > rs[k].far_) { rs[k].alive = false; continue; }
                    if (!(w.mask[k] >> s & 1)) continue;
                    double bo[64];
                    const float bd01[3] = {(rs[k].r.d.x + 1.0f) / 2.0f, (rs[k].r.d.y + 1.0f) / 2.0f, (rs[k].r.d.z + 1.0f) / 2.0f};
                    base_forward(d, contract(*sc, at(rs[k].r, tm)), bo, bd01); /* the build ray's direction (src/cache_renderer.cu:1026) */
                    const double sigma = std::exp(bo[0]);
                    double alpha = std::min(1.0, std::max(0.0, 1.0 - std::exp(-sigma * (double)dt)));
                    if (alpha > (double)sc->alpha_thre) { T *= 1.0 - alpha; ++visible; }
                    if (T < 1e-4) rs[k].alive = false;
                    w.sig[k * 8 + s] = sigma;
                    w.alpha[k * 8 + s] = alpha;
                    for (int j = 0; j < 8; ++j) w.lat[(k * 8 + s) * 8 + j] = bo[net->latent_offset + j];
                }
                rs[k].T = T;
            }
            w.need = visible > 0;
        });
        /* deterministic slot assignment (tile order within the iteration) and fill */
        for (int t : alive_list) n_samples += work[t].n_steps;  /* emitted and evaluated (:1003-1026) */
        for (int t : alive_list) {
            TileWork &w = work[t];
            const bool processed = w.n_steps > 0 && !w.sig.empty();
            if (!processed) continue;  /* reference returns early: no update */
            RayS *rs = &rays[(size_t)t * 64];
            int overflow = 0;
            if (w.need) {
                const int slot = counter++;
                overflow = slot >= capacity;
                const int tx = t % cd.bX, ty = t / cd.bX, bz = block_step[t];
                const size_t bidx = ((size_t)bz * cd.bY + ty) * cd.bX + tx;
                if (!overflow) {
                    const int sx = slot / (cd.dY * cd.dZ), sy = (slot - sx * cd.dY * cd.dZ) / cd.dZ, sz = slot - sx * cd.dY * cd.dZ - sy * cd.dZ;
                    cc->packed_index[bidx] = pack3(sx, sy, sz);
                    n_bricks[t]++;
                    for (int k = 0; k < 64; ++k)
                        for (int s = 0; s < 8; ++s) {
                            const size_t v = (size_t)slot * 512 + (size_t)s * 64 + k;
                            if (w.mask[k] >> s & 1) {
                                /* accumulateNew_cache_init_second_kernel :459-507 */
                                const double sig = w.sig[k * 8 + s];
                                const bool by_alpha = cc->variant == 1 || cc->variant == 4;
                                const double val = by_alpha ? w.alpha[k * 8 + s] : sig;
                                cc->vox_density[v] = cc->variant == 2 ? 0.0f : (float)val; /* Intermediates: slot unwritten */
                                cc->vox_isset[v] = 1.0f;
                                for (int j = 0; j < 8; ++j) cc->vox_latents[v * 8 + j] = d2h_bits(w.lat[(k * 8 + s) * 8 + j]);
                                if (cc->variant == 3 || cc->variant == 4) cc->vox_latents[v * 8] = d2h_bits(val);
                            }
                        }
                } else {
                    cc->packed_index[bidx] = -1;
                }
            }
            int n_alive = 0;
            for (int k = 0; k < 64; ++k) n_alive += rs[k].alive;
            block_step[t] += overflow ? 0 : 1;
            alive_tile[t] = !overflow && n_alive > 0;
            w.sig.clear();
        }
    }
    /* writeImageBuffer_cache_init_kernel2, :530-569: known_ranges_to */
    for (int t = 0; t < nT; ++t) {
        const int tx = t % cd.bX, ty = t / cd.bX;
        const float tr = t_from_step(*st, (float)(block_step[t] * 8) + st->near_i);
        for (int k = 0; k < 64; ++k) {
            const int px = tx * 8 + (k % 8), py = ty * 8 + (k / 8);
            if (px < cd.fW && py < cd.fH) cc->known_ranges[(size_t)py * cd.fW + px] = tr;
        }
    }
    int set = 0;
    for (int t = 0; t < nT; ++t) set += n_bricks[t];
    cc->n_bricks_set = set;
    cc->n_demanded = counter;
    cc->n_iterations = iter;
    cc->n_samples = n_samples;
    return 0;
}

/* Per-ray cache fill: CacheRenderer::initCache and its kernels
 * (src/cache_renderer.cu:571-928, sample_common_kernel src/renderer.cu:
 * 192-245).  Every cache-camera ray that hits the scene box marches in
 * sub-iterations of TARGET_BATCH_SIZE / alive (1..8) occupied samples; per
 * sub-iteration the bricks of visible samples are marked (unclamped density,
 * until T < 1e-4), new bricks get slots in (brick column, depth) order (the
 * reference's atomicAdd order is unspecified), and the voxels are written
 * (density clamped to exp(10)); a sample whose brick has no slot, or lies
 * beyond the frustum depth, ends its ray at t0, T < 1e-4 at t1.
 * known_ranges_to = the termination depth, StepsizeInfo::far for rays that
 * end otherwise.  cc->n_samples counts the padded batches as the reference. */
int orc_cache_build_per_ray(const OrcNet *net, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                            OrcCache *cc, int n_threads)
{
    NetD d; prepare_net(net, d);
    const OrcCacheDims &cd = cc->dims;
    const int W = cam->W, H = cam->H;
    const int capacity = cd.dX * cd.dY * cd.dZ;
    const size_t n_bricks = (size_t)cd.bX * cd.bY * cd.bZ, plane = (size_t)cd.bX * cd.bY;
    std::fill(cc->packed_index, cc->packed_index + n_bricks, -1);
    std::vector<uint8_t> flag(n_bricks, 0), set(n_bricks, 0);
    for (int i = 0; i < W * H; ++i) cc->known_ranges[i] = st->far_;
    struct R { Ray r; int id; float far_, t1; double T; bool done; };
    std::vector<R> alive;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            R q;
            q.r = generate_ray(*cam, x, y);
            float tn, tf;
            if (!ray_aabb(q.r, sc->aabb_from, sc->aabb_to, tn, tf)) continue;
            q.id = y * W + x;
            q.far_ = fminf(tf, st->far_);
            q.t1 = valid_t_from_t(*st, tn) + 0.0f;
            q.T = 1.0;
            q.done = false;
            alive.push_back(q);
        }
    auto brick_of = [&](int id, float tm, int &bin) -> long long {
        bin = (int)floorf(step_from_t(*st, tm) - st->near_i);
        const int bz = bin >> 3;
        if (bin < 0 || bz >= cd.bZ) return -1;
        const int x = id % W, y = id / W;
        return ((long long)bz * cd.bY + (y >> 3)) * cd.bX + (x >> 3);
    };
    long long counter = 0, n_samples = 0;
    int iter = 0;
    struct S { float t0; double lat[8], logd; };
    for (; iter < 1000 && !alive.empty(); ++iter) {
        const int n_alive = (int)alive.size();
        const int n_steps = std::min(8, std::max(1, (1 << 21) / n_alive));
        n_samples += ((long long)n_alive * n_steps + 255) / 256 * 256;
        std::vector<std::vector<S>> smp(n_alive);
        /* sample_common_kernel + inferenceLatents */
        parallel_rows(n_alive, n_threads, [&](int i) {
            R &q = alive[i];
            while ((int)smp[i].size() < n_steps) {
                const float t0 = q.t1, dt = calc_step(*st, t0), t1 = t0 + dt, tm = (t0 + t1) * 0.5f;
                if (tm > q.far_) { q.done = true; break; }
                q.t1 = t1;
                if (!occupied(*sc, bits, at(q.r, tm))) continue;
                double bo[64];
                {
                    const float qd01[3] = {(q.r.d.x + 1.0f) / 2.0f, (q.r.d.y + 1.0f) / 2.0f, (q.r.d.z + 1.0f) / 2.0f};
                    base_forward(d, contract(*sc, at(q.r, tm)), bo, qd01);
                }
                S e;
                e.t0 = t0;
                e.logd = bo[0];
                for (int j = 0; j < 8; ++j) e.lat[j] = bo[net->latent_offset + j];
                smp[i].push_back(e);
            }
        });
        /* accumulate_cache_init_first_kernel */
        for (int i = 0; i < n_alive; ++i) {
            double T = alive[i].T;
            for (const S &e : smp[i]) {
                const float dt = calc_step(*st, e.t0), tm = (e.t0 + (e.t0 + dt)) * 0.5f;
                const double alpha = std::min(1.0, std::max(0.0, 1.0 - std::exp(-std::exp(e.logd) * (double)dt)));
                if (alpha > (double)sc->alpha_thre) {
                    T *= 1.0 - alpha;
                    int bin;
                    const long long b = brick_of(alive[i].id, tm, bin);
                    if (b < 0) break;
                    flag[b] = 1;
                }
                if (T < 1e-4) break;
            }
        }
        /* reserveNewBricks_kernel, in (column, depth) order */
        for (size_t c = 0; c < plane; ++c)
            for (int z = 0; z < cd.bZ; ++z) {
                const size_t b = (size_t)z * plane + c;
                if (!flag[b]) continue;
                flag[b] = 0;
                if (set[b]) continue;
                const long long slot = counter++;
                if (slot < capacity) {
                    const int sx = (int)(slot / (cd.dY * cd.dZ)), sy = (int)((slot - (long long)sx * cd.dY * cd.dZ) / cd.dZ);
                    const int sz = (int)(slot - (long long)sx * cd.dY * cd.dZ - (long long)sy * cd.dZ);
                    cc->packed_index[b] = pack3(sx, sy, sz);
                    set[b] = 1;
                } else {
                    cc->packed_index[b] = -1;
                }
            }
        /* accumulate_cache_init_second_kernel */
        std::vector<R> next;
        for (int i = 0; i < n_alive; ++i) {
            R &q = alive[i];
            double T = q.T;
            float term = st->far_;
            bool live = !q.done;
            for (const S &e : smp[i]) {
                const float dt = calc_step(*st, e.t0), t1 = e.t0 + dt, tm = (e.t0 + t1) * 0.5f;
                const double density = std::exp(std::min(e.logd, 10.0));
                const double alpha = std::min(1.0, std::max(0.0, 1.0 - std::exp(-density * (double)dt)));
                if (alpha > (double)sc->alpha_thre) {
                    T *= 1.0 - alpha;
                    int bin;
                    const long long b = brick_of(q.id, tm, bin);
                    const int packed = b >= 0 ? cc->packed_index[b] : -1;
                    if (packed < 0) { live = false; term = e.t0; break; }
                    const int slot = ((packed >> 20) & 1023) * cd.dY * cd.dZ + ((packed >> 10) & 1023) * cd.dZ + (packed & 1023);
                    const int x = q.id % W, y = q.id / W;
                    const size_t v = (size_t)slot * 512 + (size_t)(bin & 7) * 64 + (y & 7) * 8 + (x & 7);
                    const bool by_alpha = cc->variant == 1 || cc->variant == 4;
                    const double val = by_alpha ? alpha : density;
                    cc->vox_density[v] = cc->variant == 2 ? 0.0f : (float)val;
                    cc->vox_isset[v] = 1.0f;
                    for (int j = 0; j < 8; ++j) cc->vox_latents[v * 8 + j] = d2h_bits(e.lat[j]);
                    if (cc->variant == 3 || cc->variant == 4) cc->vox_latents[v * 8] = d2h_bits(val);
                }
                if (T < 1e-4) { live = false; term = t1; break; }
            }
            q.T = T;
            if (live) next.push_back(q);
            else cc->known_ranges[q.id] = term;
        }
        alive.swap(next);
    }
    cc->n_demanded = (int)counter;
    cc->n_bricks_set = (int)std::min<long long>(counter, capacity);
    cc->n_iterations = iter;
    cc->n_samples = n_samples;
    return 0;
}

/* voxel lookup through the data array's texel addressing (tex3D point with
 * border addressing, include/util/cuda_readwrite_array.h:41-62) */
struct Vox { double density, isset, lat[8]; };
inline bool fetch_texel(const OrcCache &cc, int X, int Y, int Z, Vox &v)
{
    const OrcCacheDims &cd = cc.dims;
    if (X < 0 || Y < 0 || Z < 0 || X >= cd.dX * 8 || Y >= cd.dY * 8 || Z >= cd.dZ * 8) return false;
    const int slot = (X / 8) * cd.dY * cd.dZ + (Y / 8) * cd.dZ + (Z / 8);
    const size_t i = (size_t)slot * 512 + (size_t)(Z % 8) * 64 + (Y % 8) * 8 + (X % 8);
    v.density = cc.vox_density[i]; v.isset = cc.vox_isset[i];
    for (int j = 0; j < 8; ++j) v.lat[j] = h2d(cc.vox_latents[i * 8 + j]);
    return true;
}

inline int brick_lookup(const OrcCache &cc, int bx, int by, int bz)
{
    const OrcCacheDims &cd = cc.dims;
    return cc.packed_index[((size_t)bz * cd.bY + by) * cd.bX + bx];
}

/* CacheBasicRenderer's cache decision and lookup at froxel point fp
 * (sample_cache_kernel, src/cache_basic_renderer.cu:95-210; froxel2data and
 * fetchBrickTex3DInterpol, include/raymarch_common.h:331-444): 1 cache
 * (lat = head inputs, sigma = density), or 2 dropped with the reason in the
 * upper bits (5 brick without a slot, 6 voxel not set, 7 alpha not above the
 * threshold).  Texture weights in full precision (the texture unit's 8-bit
 * weights are not emulated). */
int basic_sample(const OrcCache &cc, const OrcScene *sc, V3 fp, float dt, double *lat, double &sigma)
{
    const OrcCacheDims &cd = cc.dims;
    const int bx = (int)(fp.x / 8.0f), by = (int)(fp.y / 8.0f), bz = (int)(fp.z / 8.0f);
    float ix = fp.x - (float)(bx * 8), iy = fp.y - (float)(by * 8), iz = fp.z - (float)(bz * 8);
    bool inside_brick = true;
    if (cc.inter_brick) {
        inside_brick = ix >= 0.5f && ix < 7.5f && iy >= 0.5f && iy < 7.5f && iz >= 0.5f && iz < 7.5f;
    } else {
        ix = std::min(std::max(ix, 0.5f), 7.5f);
        iy = std::min(std::max(iy, 0.5f), 7.5f);
        iz = std::min(std::max(iz, 0.5f), 7.5f);
    }
    const int packed = brick_lookup(cc, bx, by, bz);
    if (packed < 0) return 2 | (5 << 2);
    const float dx = (float)(((packed >> 20) & 1023) * 8) + ix, dy = (float)(((packed >> 10) & 1023) * 8) + iy,
                dz = (float)((packed & 1023) * 8) + iz;
    Vox v0;
    if (!fetch_texel(cc, (int)floorf(dx), (int)floorf(dy), (int)floorf(dz), v0) || !(v0.isset > 0.0)) return 2 | (6 << 2);
    double weight = 0, dac = 0, ls[8] = {0};
    auto add = [&](const Vox &v, double w) {
        weight += w * v.isset; dac += w * v.density;
        for (int j = 0; j < 8; ++j) ls[j] += w * v.lat[j];
    };
    if (cc.interp == 3) {
        add(v0, 1.0);
    } else if (cc.interp == 0 && inside_brick) { /* tex3D linear inside the data array */
        const float ax = dx - 0.5f, ay = dy - 0.5f, az = dz - 0.5f;
        const float x0 = floorf(ax), y0 = floorf(ay), z0 = floorf(az);
        const double l[3] = {(double)(ax - x0), (double)(ay - y0), (double)(az - z0)};
        for (int c = 0; c < 8; ++c) {
            const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
            const double w = (ox ? l[0] : 1.0 - l[0]) * (oy ? l[1] : 1.0 - l[1]) * (oz ? l[2] : 1.0 - l[2]);
            Vox v;
            if (fetch_texel(cc, (int)x0 + ox, (int)y0 + oy, (int)z0 + oz, v)) add(v, w);
        }
    } else { /* 8 froxel corners, each through its own brick */
        const float fx0 = floorf(fp.x - 0.5f), fy0 = floorf(fp.y - 0.5f), fz0 = floorf(fp.z - 0.5f);
        const double l[3] = {(double)interp_fn(fp.x - 0.5f - fx0, cc.interp), (double)interp_fn(fp.y - 0.5f - fy0, cc.interp),
                             (double)interp_fn(fp.z - 0.5f - fz0, cc.interp)};
        for (int c = 0; c < 8; ++c) {
            const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
            const double w = (ox ? l[0] : 1.0 - l[0]) * (oy ? l[1] : 1.0 - l[1]) * (oz ? l[2] : 1.0 - l[2]);
            const float cx = fx0 + (float)ox, cy = fy0 + (float)oy, cz = fz0 + (float)oz;
            if (!(cx >= 0 && cx < (float)cd.fW && cy >= 0 && cy < (float)cd.fH && cz >= 0 && cz < (float)cd.fD)) continue;
            const int cbx = (int)(cx / 8.0f), cby = (int)(cy / 8.0f), cbz = (int)(cz / 8.0f);
            const int pk = brick_lookup(cc, cbx, cby, cbz);
            if (pk < 0) continue;
            Vox v;
            if (fetch_texel(cc, ((pk >> 20) & 1023) * 8 + ((int)cx - cbx * 8), ((pk >> 10) & 1023) * 8 + ((int)cy - cby * 8),
                            (pk & 1023) * 8 + ((int)cz - cbz * 8), v))
                add(v, w);
        }
    }
    double alpha, density;
    switch (cc.variant) {
    case 1: alpha = dac; density = -std::log(std::max(1.0 - alpha, 1e-6)) / dt; break;
    case 2: density = std::exp(ls[0] / weight); alpha = std::min(1.0, std::max(0.0, 1.0 - std::exp(-density * dt))); break;
    case 3: density = ls[0]; alpha = std::min(1.0, std::max(0.0, 1.0 - std::exp(-density * dt))); ls[0] = std::log(density); break;
    case 4: alpha = ls[0]; density = -std::log(std::max(1.0 - alpha, 1e-6)) / dt; ls[0] = std::log(density); break;
    default: density = dac; alpha = std::min(1.0, std::max(0.0, 1.0 - std::exp(-density * dt))); break;
    }
    if (cc.reweight && cc.keep_first) ls[0] *= weight;
    if (!(alpha > (double)sc->alpha_thre)) return 2 | (7 << 2);
    const double div = cc.reweight ? weight : 1.0;
    for (int j = 0; j < 8; ++j) lat[j] = ls[j] / div;
    sigma = density;
    return 1;
}

/* Front-to-back compositing of given network outputs over one batch, as
 * accumulate_performance_kernel (src/performance_renderer.cu:71-125): ray i
 * owns samples s = 0 .. n_steps[i]-1 at row s * n_alive + i (sample-major),
 * out4 holds 4 rows of `batch` values (r, g, b logits and log-density, the
 * fp16 outputs as floats), t0 the samples' t0; results (rgb, T) and alive
 * are updated in place (alive cleared when T < 1e-4), with the oracle's
 * float64 compositing step. */
void orc_composite_rows(int n_alive, int batch, const OrcSteps *st, float alpha_thre, const int32_t *n_steps, uint8_t *alive,
                        float *results, const float *out4, const float *t0)
{
    for (int i = 0; i < n_alive; ++i) {
        double rgb[3] = {results[4 * i], results[4 * i + 1], results[4 * i + 2]}, T = results[4 * i + 3];
        for (int s = 0; s < n_steps[i]; ++s) {
            const size_t row = (size_t)s * n_alive + i;
            const double lg[3] = {out4[row], out4[row + (size_t)batch], out4[row + 2 * (size_t)batch]};
            const double sigma = std::exp((double)out4[row + 3 * (size_t)batch]);
            if (composite(sigma, lg, calc_step(*st, t0[row]), alpha_thre, rgb, T)) {
                alive[i] = 0;
                break;
            }
        }
        for (int k = 0; k < 3; ++k) results[4 * i + k] = (float)rgb[k];
        results[4 * i + 3] = (float)T;
    }
}

/* Cached render: CachePerformanceRenderer::render and its kernels
 * (src/cache_performance_renderer.cu:22-313, 678-908, 1059-1263) as one pass
 * per ray.  counts[4*W*H]: resample, cache, dropped, steps.  reasons[8]
 * (optional): over the samples composited or dropped, why they were not
 * cache hits: 1 outside the cache image, 2 outside the froxel depth, 3 before
 * the near plane, 4 beyond the known range (resampled); 5 brick without a
 * slot, 6 empty voxel (not set: basic), 7 alpha (basic) (dropped). */
int orc_render_cached(const OrcNet *net, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                      const OrcCache *cc, const OrcCam *ccam, const OrcSteps *cst, int mode,
                      int row0, int row1, float *results, int32_t *counts, int n_threads, long long *reasons,
                      double *contrib)
{
    NetD d; prepare_net(net, d);
    const OrcCacheDims &cd = cc->dims;
    const int W = cam->W;
    std::mutex reason_mutex;
    parallel_rows(row1 - row0, n_threads, [&](int rr) {
        const int y = row0 + rr;
        long long why_row[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int x = 0; x < W; ++x) {
            const size_t id = (size_t)y * W + x;
            const Ray r = generate_ray(*cam, x, y);
            float tn, tf;
            const bool hits = ray_aabb(r, sc->aabb_from, sc->aabb_to, tn, tf);
            double rgb[3] = {0, 0, 0}, T = 1.0, w_contrib[2] = {0.0, 0.0};
            int n_res = 0, n_cache = 0, n_drop = 0, nst = 0;
            if (hits) {
                const Ray rc = transform_ray(r, ccam->w2c);
                const float far_ = fminf(tf, st->far_);
                float t1 = start_t1(*cam, *st, tn, (int)id);
                const float d01[3] = {(r.d.x + 1.0f) / 2.0f, (r.d.y + 1.0f) / 2.0f, (r.d.z + 1.0f) / 2.0f};
                for (;;) {
                    const float t0 = t1;
                    const float dt = calc_step(*st, t0);
                    t1 = t0 + dt;
                    const float tm = (t0 + t1) * 0.5f;
                    ++nst;
                    if (tm > far_) break;
                    const V3 wp = at(r, tm);
                    if (!occupied(*sc, bits, wp)) continue;
                    /* classification, sample_cache_performance_kernel :91-163 */
                    float tfr;
                    const V3 fp = cam2froxel(at(rc, tm), *ccam, *cst, tfr);
                    const bool in_fov = fp.x >= 0 && fp.x < (float)cd.fW && fp.y >= 0 && fp.y < (float)cd.fH;
                    const bool inside = in_fov && fp.z >= 0 && fp.z < (float)cd.fD;
                    bool unsampled = true;
                    float kr = 0.0f;
                    if (in_fov) {
                        kr = cc->known_ranges[(size_t)(int)floorf(fp.y) * cd.fW + (int)floorf(fp.x)];
                        unsampled = tfr < cst->near_ || tfr > kr;
                    }
                    /* why the sample is outside the cache's sampled region (0: inside): the first failing
                     * test in the order image, near plane, known range, froxel depth */
                    const int why_out = !in_fov ? 1 : tfr < cst->near_ ? 3 : tfr > kr ? 4 : !inside ? 2 : 0;
                    int kind = 0; /* 0 resample, 1 cache, 2 drop */
                    double blat[8], bsigma = 0.0;
                    if (cc->basic) {
                        /* CacheBasicRenderer: decided and looked up at the midpoint */
                        const int code = (!inside || unsampled) ? 0 : basic_sample(*cc, sc, fp, dt, blat, bsigma);
                        kind = code & 3;
                        if (kind == 0) ++why_row[why_out];
                        if (kind == 2) { ++why_row[code >> 2]; ++n_drop; continue; }
                    } else if (!inside || unsampled) {
                        if (mode == 1) continue;
                        kind = 0;
                        ++why_row[why_out];
                    } else {
                        if (mode == 2) continue;
                        const int bx = (int)(fp.x / 8.0f), by = (int)(fp.y / 8.0f), bz = (int)(fp.z / 8.0f);
                        const int packed = brick_lookup(*cc, bx, by, bz);
                        kind = 2;
                        int why_drop = 5;
                        if (packed >= 0) {
                            why_drop = 6;
                            const float ix = fp.x - (float)(bx * 8), iy = fp.y - (float)(by * 8), iz = fp.z - (float)(bz * 8);
                            const float ax = (float)(((packed >> 20) & 1023) * 8) + ix;
                            const float ay = (float)(((packed >> 10) & 1023) * 8) + iy;
                            const float az = (float)((packed & 1023) * 8) + iz;
                            Vox v;
                            if (fetch_texel(*cc, (int)floorf(ax), (int)floorf(ay), (int)floorf(az), v) && v.density > 0.0) kind = 1;
                        }
                        if (kind == 2) { ++why_row[why_drop]; ++n_drop; continue; }
                    }
                    const float tmh = cc->basic ? tm : t0 + dt * 0.5f;  /* generateNetworkInput_* :234, :287 */
                    /* a view-dependent head's initial direction for a cache sample: from the cache camera to
                     * the sample (src/cache_performance_renderer.cu:290-312, src/cache_basic_renderer.cu:86-87) */
                    float init01[3];
                    {
                        const V3 wp = at(r, tmh);
                        const double vx = (double)wp.x - ccam->c2w[3], vy = (double)wp.y - ccam->c2w[7], vz = (double)wp.z - ccam->c2w[11];
                        const double nv = std::sqrt(vx * vx + vy * vy + vz * vz);
                        init01[0] = (float)((vx / nv + 1.0) / 2.0);
                        init01[1] = (float)((vy / nv + 1.0) / 2.0);
                        init01[2] = (float)((vz / nv + 1.0) / 2.0);
                    }
                    double sigma, lg[3];
                    const V3 cp = contract(*sc, at(r, tmh)); /* the head's network input position */
                    if (kind == 1 && cc->basic) {
                        head_forward(d, blat, d01, lg, init01, &cp);
                        sigma = bsigma;
                        ++n_cache;
                    } else if (kind == 0) {
                        double bo[64];
                        base_forward(d, cp, bo, d01);
                        head_forward(d, bo + net->latent_offset, d01, lg, nullptr, &cp);
                        sigma = std::exp(bo[0]);
                        ++n_res;
                    } else {
                        /* generateNetworkInput_cache_shfl_perf_kernel_cg :678-787 */
                        float tfr2;
                        const V3 f2 = cam2froxel(at(rc, tmh), *ccam, *cst, tfr2);
                        const float fx0 = floorf(f2.x - 0.5f), fy0 = floorf(f2.y - 0.5f), fz0 = floorf(f2.z - 0.5f);
                        const double lt[3] = {(double)interp_fn(f2.x - 0.5f - fx0, cc->interp),
                                              (double)interp_fn(f2.y - 0.5f - fy0, cc->interp),
                                              (double)interp_fn(f2.z - 0.5f - fz0, cc->interp)};
                        double wsum = 0, dsum = 0, lsum[8] = {0};
                        for (int c = 0; c < 8; ++c) {
                            const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
                            const double w = (ox ? lt[0] : 1.0 - lt[0]) * (oy ? lt[1] : 1.0 - lt[1]) * (oz ? lt[2] : 1.0 - lt[2]);
                            const float cx = fx0 + (float)ox, cy = fy0 + (float)oy, cz = fz0 + (float)oz;
                            const bool fov = cx >= 0 && cx < (float)cd.fW && cy >= 0 && cy < (float)cd.fH;
                            if (!(fov && cz >= 0 && cz < (float)cd.fD)) continue;
                            const int bx = (int)(cx / 8.0f), by = (int)(cy / 8.0f), bz = (int)(cz / 8.0f);
                            const int packed = brick_lookup(*cc, bx, by, bz);
                            if (packed < 0) continue;
                            const int X = ((packed >> 20) & 1023) * 8 + ((int)cx - bx * 8);
                            const int Y = ((packed >> 10) & 1023) * 8 + ((int)cy - by * 8);
                            const int Z = (packed & 1023) * 8 + ((int)cz - bz * 8);
                            Vox v;
                            if (!fetch_texel(*cc, X, Y, Z, v)) continue;
                            wsum += w * v.isset; dsum += w * v.density;
                            for (int j = 0; j < 8; ++j) lsum[j] += w * v.lat[j];
                        }
                        double lat[8];
                        for (int j = 0; j < 8; ++j) lat[j] = lsum[j] / wsum;
                        if (cc->variant == 3) {
                            /* DensityIntermediates (:776-781): latent 0 is the density,
                             * log(sum w density) enters the head and gives sigma */
                            lat[0] = net->mimic_fp16 ? round_h(std::log(lsum[0])) : std::log(lsum[0]);
                            head_forward(d, lat, d01, lg, init01, &cp);
                            sigma = std::exp(lat[0]);
                        } else {
                            head_forward(d, lat, d01, lg, init01, &cp);
                            sigma = std::max(dsum, 1e-6);
                        }
                        ++n_cache;
                    }
                    const double T_before = T;
                    const bool stop = composite(sigma, lg, dt, sc->alpha_thre, rgb, T);
                    /* contribution weight alpha T of the sample (accumulate_cache_perf_kernel<DEBUG>, :867-871) */
                    if (T != T_before) w_contrib[kind == 1 ? 1 : 0] += T_before - T;
                    if (stop) break;
                }
            }
            results[4 * id + 0] = (float)rgb[0]; results[4 * id + 1] = (float)rgb[1];
            results[4 * id + 2] = (float)rgb[2]; results[4 * id + 3] = (float)T;
            if (contrib) { contrib[2 * id] = w_contrib[0]; contrib[2 * id + 1] = w_contrib[1]; }
            if (counts) { counts[4 * id] = n_res; counts[4 * id + 1] = n_cache; counts[4 * id + 2] = n_drop; counts[4 * id + 3] = nst; }
        }
        if (reasons) {
            std::lock_guard<std::mutex> lk(reason_mutex);
            for (int q = 0; q < 8; ++q) reasons[q] += why_row[q];
        }
    });
    return 0;
}


}  /* extern "C" */

/* ========================================================================== */
/* Differentiable render: L2 loss of the plain render at a list of pixels and
 * its adjoint with respect to the hash table and both MLPs (float64).
 *
 * Loss: L = (1/N) sum_rays sum_k (C_k + T - target_k)^2, the white-background
 * pixel of the plain render (writeImageBuffer_performance_kernel,
 * src/performance_renderer.cu:127-149, before the 8-bit conversion).
 * Compositing adjoint, in sample order without division: with g = dL/dC,
 * g_T = dL/dT, X_total = g.C + g_T T_final and X_i the prefix sum of
 * T_j alpha_j g.c_j over used samples j <= i,
 *   dL/dsigma_i = dt_i (T_{i+1} g.c_i - (X_total - X_i)),
 *   dL/dc_i     = T_i alpha_i g;
 * samples skipped by the alpha threshold carry no gradient, and the early
 * termination (T < 1e-4) ends both passes at the same sample.  The network
 * adjoint treats the fp16 rounding of activations (mimic_fp16) as identity;
 * ReLU passes gradient where its output is > 0.
 * Parameter blobs (and gradients) use the model file layouts: table
 * [entries x F]; base [width x enc_w_pad][base_out_pad x width]; head
 * [width x head_in_pad][width x width]*[16 x width].                         */
/* ========================================================================== */
namespace {

struct Acts {
    double feat[64], h1[128], out2[64], in[128], hid[4][128], out[16];
};

void forward_acts(const NetD &d, V3 pos, const float *d01, Acts &A)
{
    const OrcNet &n = *d.n;
    hash_encode(d, pos, A.feat);
    dense_layer(d.bw0.data(), n.width, n.enc_w_pad, A.feat, A.h1, true, n.mimic_fp16);
    dense_layer(d.bw1.data(), n.base_out_pad, n.width, A.h1, A.out2, false, n.mimic_fp16);
    for (int i = 0; i < n.n_latents; ++i) A.in[i] = A.out2[n.latent_offset + i];
    sh16(d01, A.in + n.n_latents);
    if (n.mimic_fp16) for (int i = n.n_latents; i < n.n_latents + 16; ++i) A.in[i] = round_h(A.in[i]);
    for (int i = n.head_in; i < n.head_in_pad; ++i) A.in[i] = 1.0;
    dense_layer(d.hw[0].data(), n.width, n.head_in_pad, A.in, A.hid[0], true, n.mimic_fp16);
    for (int l = 1; l < n.head_layers - 1; ++l)
        dense_layer(d.hw[l].data(), n.width, n.width, A.hid[l - 1], A.hid[l], true, n.mimic_fp16);
    dense_layer(d.hw[n.head_layers - 1].data(), 16, n.width, A.hid[n.head_layers - 2], A.out, false, n.mimic_fp16);
}

/* y = W x (W: out x in) backward: gW += dy (x) x, dx = W^T dy (dx may be null) */
inline void dense_backward(const double *W, int out, int in, const double *x, const double *dy, double *gW, double *dx)
{
    if (dx) for (int i = 0; i < in; ++i) dx[i] = 0.0;
    for (int o = 0; o < out; ++o) {
        const double g = dy[o];
        if (g == 0.0) continue;
        const double *w = W + (size_t)o * in;
        if (gW) { double *gw = gW + (size_t)o * in; for (int i = 0; i < in; ++i) gw[i] += g * x[i]; }
        if (dx) for (int i = 0; i < in; ++i) dx[i] += g * w[i];
    }
}

/* hash-grid adjoint: scatter dfeat into the table gradient with the trilinear weights */
void hash_backward(const NetD &d, V3 pos, const double *dfeat, double *g_table)
{
    const OrcNet &n = *d.n;
    const float px[3] = {pos.x, pos.y, pos.z};
    for (int l = 0; l < n.n_levels; ++l) {
        uint32_t g[3]; double fr[3];
        for (int k = 0; k < 3; ++k) {
            const float p = fmaf(n.scale[l], px[k], 0.5f);
            const float fl = floorf(p);
            g[k] = (uint32_t)(int)fl;
            fr[k] = (double)(p - fl);
        }
        for (int c = 0; c < 8; ++c) {
            uint32_t q[3]; double w = 1.0;
            for (int k = 0; k < 3; ++k) {
                const int b = (c >> k) & 1;
                q[k] = g[k] + (uint32_t)b;
                w *= b ? fr[k] : 1.0 - fr[k];
            }
            uint32_t idx;
            if (n.dense[l]) idx = q[0] + q[1] * n.res[l] + q[2] * n.res[l] * n.res[l];
            else idx = (q[0] * 1u) ^ (q[1] * 2654435761u) ^ (q[2] * 805459861u);
            idx %= n.size[l];
            double *e = &g_table[((size_t)n.offset[l] + idx) * n.F];
            for (int f = 0; f < n.F; ++f) e[f] += w * dfeat[l * n.F + f];
        }
    }
}

/* head forward from given latents (the cached path's head input) */
void forward_head_acts(const NetD &d, const double *lat, const float *d01, Acts &A)
{
    const OrcNet &n = *d.n;
    for (int i = 0; i < n.n_latents; ++i) A.in[i] = lat[i];
    sh16(d01, A.in + n.n_latents);
    if (n.mimic_fp16) for (int i = n.n_latents; i < n.n_latents + 16; ++i) A.in[i] = round_h(A.in[i]);
    for (int i = n.head_in; i < n.head_in_pad; ++i) A.in[i] = 1.0;
    dense_layer(d.hw[0].data(), n.width, n.head_in_pad, A.in, A.hid[0], true, n.mimic_fp16);
    for (int l = 1; l < n.head_layers - 1; ++l)
        dense_layer(d.hw[l].data(), n.width, n.width, A.hid[l - 1], A.hid[l], true, n.mimic_fp16);
    dense_layer(d.hw[n.head_layers - 1].data(), 16, n.width, A.hid[n.head_layers - 2], A.out, false, n.mimic_fp16);
}

/* head adjoint: weight gradients into g_head, dL/d(head input) into din */
void head_backward(const NetD &d, const Acts &A, const double *d_logit, double *g_head, double *din)
{
    const OrcNet &n = *d.n;
    double dy[128];
    for (int i = 0; i < 16; ++i) dy[i] = i < 3 ? d_logit[i] : 0.0;
    size_t head_off[4], off = 0;
    for (int l = 0; l < n.head_layers; ++l) {
        head_off[l] = off;
        off += (size_t)(l == 0 ? n.head_in_pad : n.width) * (l == n.head_layers - 1 ? 16 : n.width);
    }
    const int L = n.head_layers;
    dense_backward(d.hw[L - 1].data(), 16, n.width, A.hid[L - 2], dy, g_head ? g_head + head_off[L - 1] : nullptr, din);
    for (int l = L - 2; l >= 0; --l) {
        for (int i = 0; i < n.width; ++i) dy[i] = A.hid[l][i] > 0.0 ? din[i] : 0.0;
        const int in = l == 0 ? n.head_in_pad : n.width;
        const double *x = l == 0 ? A.in : A.hid[l - 1];
        dense_backward(d.hw[l].data(), n.width, in, x, dy, g_head ? g_head + head_off[l] : nullptr, din);
    }
}

/* network adjoint of one sample given dL/d(log sigma) and dL/d(rgb logits) */
void network_backward(const NetD &d, V3 pos, const Acts &A, double d_logsigma, const double *d_logit,
                      double *g_table, double *g_base, double *g_head)
{
    const OrcNet &n = *d.n;
    double dy[128], dx[128];
    for (int i = 0; i < 16; ++i) dy[i] = i < 3 ? d_logit[i] : 0.0;
    /* head, last layer back to its first */
    size_t head_off[4], off = 0;
    for (int l = 0; l < n.head_layers; ++l) {
        head_off[l] = off;
        off += (size_t)(l == 0 ? n.head_in_pad : n.width) * (l == n.head_layers - 1 ? 16 : n.width);
    }
    const int L = n.head_layers;
    dense_backward(d.hw[L - 1].data(), 16, n.width, A.hid[L - 2], dy, g_head ? g_head + head_off[L - 1] : nullptr, dx);
    for (int l = L - 2; l >= 0; --l) {
        for (int i = 0; i < n.width; ++i) dy[i] = A.hid[l][i] > 0.0 ? dx[i] : 0.0;
        const int in = l == 0 ? n.head_in_pad : n.width;
        const double *x = l == 0 ? A.in : A.hid[l - 1];
        dense_backward(d.hw[l].data(), n.width, in, x, dy, g_head ? g_head + head_off[l] : nullptr, dx);
    }
    /* density network */
    double dout2[64];
    for (int i = 0; i < n.base_out_pad; ++i) dout2[i] = 0.0;
    dout2[0] += d_logsigma;
    for (int j = 0; j < n.n_latents; ++j) dout2[n.latent_offset + j] += dx[j];
    const size_t nb0 = (size_t)n.width * n.enc_w_pad;
    double dh[128];
    dense_backward(d.bw1.data(), n.base_out_pad, n.width, A.h1, dout2, g_base ? g_base + nb0 : nullptr, dh);
    for (int i = 0; i < n.width; ++i) dh[i] = A.h1[i] > 0.0 ? dh[i] : 0.0;
    double dfeat[64];
    dense_backward(d.bw0.data(), n.width, n.enc_w_pad, A.feat, dh, g_base, dfeat);
    if (g_table) hash_backward(d, pos, dfeat, g_table);
}

void apply_perturbations(NetD &d, const int32_t *group, const int64_t *index, const double *delta, int n)
{
    for (int i = 0; i < n; ++i) {
        size_t k = (size_t)index[i];
        if (group[i] == 0) { d.table[k] += delta[i]; continue; }
        if (group[i] == 1) {
            if (k < d.bw0.size()) d.bw0[k] += delta[i];
            else d.bw1[k - d.bw0.size()] += delta[i];
            continue;
        }
        for (int l = 0; l < d.n->head_layers; ++l) {
            if (k < d.hw[l].size()) { d.hw[l][k] += delta[i]; break; }
            k -= d.hw[l].size();
        }
    }
}

/* one ray of the differentiable render: forward, then (if grads) the adjoint */
double ray_loss_grad(const NetD &d, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                     int px, int py, const float *target, double inv_n, double *pred,
                     double *g_table, double *g_base, double *g_head)
{
    const OrcNet &n = *d.n;
    const Ray r = generate_ray(*cam, px, py);
    float tn, tf;
    struct S { V3 pos; float dt; };
    std::vector<S> samples;
    std::vector<double> sig, rgbv;
    double C[3] = {0, 0, 0}, T = 1.0;
    const float d01[3] = {(r.d.x + 1.0f) / 2.0f, (r.d.y + 1.0f) / 2.0f, (r.d.z + 1.0f) / 2.0f};
    if (ray_aabb(r, sc->aabb_from, sc->aabb_to, tn, tf)) {
        const float far_ = fminf(tf, st->far_);
        float t1 = start_t1(*cam, *st, tn, py * cam->W + px);
        for (;;) {
            const float t0 = t1;
            const float dt = calc_step(*st, t0);
            t1 = t0 + dt;
            const float tm = (t0 + t1) * 0.5f;
            if (tm > far_) break;
            const V3 wp = at(r, tm);
            if (!occupied(*sc, bits, wp)) continue;
            const V3 cp = contract(*sc, wp);
            Acts A;
            forward_acts(d, cp, d01, A);
            const double sigma = std::exp(A.out2[0]);
            samples.push_back({cp, dt});
            sig.push_back(sigma);
            for (int k = 0; k < 3; ++k) rgbv.push_back(sigmoid(A.out[k]));
            if (composite(sigma, A.out, dt, sc->alpha_thre, C, T)) break;
        }
    }
    double loss = 0.0, g[3];
    for (int k = 0; k < 3; ++k) {
        const double e = C[k] + T - (double)target[k];
        loss += e * e * inv_n;
        g[k] = 2.0 * e * inv_n;
    }
    if (pred) { pred[0] = C[0]; pred[1] = C[1]; pred[2] = C[2]; pred[3] = T; }
    if (!(g_table || g_base || g_head)) return loss;
    const double gT = g[0] + g[1] + g[2];
    const double x_total = g[0] * C[0] + g[1] * C[1] + g[2] * C[2] + gT * T;
    double Ti = 1.0, x_prefix = 0.0;
    for (size_t i = 0; i < samples.size(); ++i) {
        const double sigma = sig[i];
        const double *c = &rgbv[3 * i];
        double alpha = 1.0 - std::exp(-sigma * (double)samples[i].dt);
        alpha = std::min(1.0, std::max(0.0, alpha));
        if (!(alpha > (double)sc->alpha_thre)) continue;
        const double gc = g[0] * c[0] + g[1] * c[1] + g[2] * c[2];
        x_prefix += Ti * alpha * gc;
        const double T_next = Ti * (1.0 - alpha);
        const double d_sigma = (double)samples[i].dt * (T_next * gc - (x_total - x_prefix));
        double d_logit[3];
        for (int k = 0; k < 3; ++k) d_logit[k] = g[k] * Ti * alpha * c[k] * (1.0 - c[k]);
        Acts A;
        forward_acts(d, samples[i].pos, d01, A);
        network_backward(d, samples[i].pos, A, d_sigma * sigma, d_logit, g_table, g_base, g_head);
        Ti = T_next;
        if (Ti < 1e-4) break;
    }
    (void)n;
    return loss;
}

/* one ray of the cached differentiable render: the classification and
 * lookups of orc_render_cached with voxel latents taken from `lat`
 * (index into [slots][512][8]), then the adjoint; cache rows pass dL/dlatents
 * to their corners with weight w_c / sum(w isset).  Density voxels get no
 * gradient. */
struct LatentSource { /* the cache's fp16 latents plus perturbations (index, delta) */
    const uint16_t *lat16;
    const int64_t *pidx;
    const double *pdel;
    int npert;
    double operator()(size_t i) const
    {
        double v = h2d(lat16[i]);
        for (int k = 0; k < npert; ++k)
            if ((size_t)pidx[k] == i) v += pdel[k];
        return v;
    }
};

double ray_loss_grad_cached(const NetD &d, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                            const OrcCache *cc, const OrcCam *ccam, const OrcSteps *cst, const LatentSource &lat, int px, int py,
                            const float *target, double inv_n, double *pred, double *g_table, double *g_base, double *g_head,
                            double *g_lat)
{
    const OrcNet &n = *d.n;
    const OrcCacheDims &cd = cc->dims;
    struct S { int kind; V3 pos; float dt; double sigma; double lat[8]; int nc; size_t vi[8]; double w[8]; double wsum; };
    std::vector<S> samples;
    std::vector<double> rgbv;
    double C[3] = {0, 0, 0}, T = 1.0;
    const Ray r = generate_ray(*cam, px, py);
    const float d01[3] = {(r.d.x + 1.0f) / 2.0f, (r.d.y + 1.0f) / 2.0f, (r.d.z + 1.0f) / 2.0f};
    float tn, tf;
    if (ray_aabb(r, sc->aabb_from, sc->aabb_to, tn, tf)) {
        const Ray rc = transform_ray(r, ccam->w2c);
        const float far_ = fminf(tf, st->far_);
        float t1 = start_t1(*cam, *st, tn, py * cam->W + px);
        for (;;) {
            const float t0 = t1;
            const float dt = calc_step(*st, t0);
            t1 = t0 + dt;
            const float tm = (t0 + t1) * 0.5f;
            if (tm > far_) break;
            const V3 wp = at(r, tm);
            if (!occupied(*sc, bits, wp)) continue;
            float tfr;
            const V3 fp = cam2froxel(at(rc, tm), *ccam, *cst, tfr);
            const bool in_fov = fp.x >= 0 && fp.x < (float)cd.fW && fp.y >= 0 && fp.y < (float)cd.fH;
            const bool inside = in_fov && fp.z >= 0 && fp.z < (float)cd.fD;
            bool unsampled = true;
            if (in_fov) {
                const float kr = cc->known_ranges[(size_t)(int)floorf(fp.y) * cd.fW + (int)floorf(fp.x)];
                unsampled = tfr < cst->near_ || tfr > kr;
            }
            int kind = 0;
            if (inside && !unsampled) {
                const int bx = (int)(fp.x / 8.0f), by = (int)(fp.y / 8.0f), bz = (int)(fp.z / 8.0f);
                const int packed = brick_lookup(*cc, bx, by, bz);
                kind = 2;
                if (packed >= 0) {
                    const float ix = fp.x - (float)(bx * 8), iy = fp.y - (float)(by * 8), iz = fp.z - (float)(bz * 8);
                    const float ax = (float)(((packed >> 20) & 1023) * 8) + ix;
                    const float ay = (float)(((packed >> 10) & 1023) * 8) + iy;
                    const float az = (float)((packed & 1023) * 8) + iz;
                    Vox v;
                    if (fetch_texel(*cc, (int)floorf(ax), (int)floorf(ay), (int)floorf(az), v) && v.density > 0.0) kind = 1;
                }
                if (kind == 2) continue;
            }
            const float tmh = t0 + dt * 0.5f;
            S smp{};
            smp.kind = kind;
            smp.dt = dt;
            Acts A;
            if (kind == 0) {
                smp.pos = contract(*sc, at(r, tmh));
                forward_acts(d, smp.pos, d01, A);
                smp.sigma = std::exp(A.out2[0]);
            } else {
                float tfr2;
                const V3 f2 = cam2froxel(at(rc, tmh), *ccam, *cst, tfr2);
                const float fx0 = floorf(f2.x - 0.5f), fy0 = floorf(f2.y - 0.5f), fz0 = floorf(f2.z - 0.5f);
                const double lt[3] = {(double)interp_fn(f2.x - 0.5f - fx0, cc->interp),
                                      (double)interp_fn(f2.y - 0.5f - fy0, cc->interp),
                                      (double)interp_fn(f2.z - 0.5f - fz0, cc->interp)};
                double dsum = 0, lsum[8] = {0};
                smp.wsum = 0;
                smp.nc = 0;
                for (int c = 0; c < 8; ++c) {
                    const int ox = (c >> 2) & 1, oy = (c >> 1) & 1, oz = c & 1;
                    const double w = (ox ? lt[0] : 1.0 - lt[0]) * (oy ? lt[1] : 1.0 - lt[1]) * (oz ? lt[2] : 1.0 - lt[2]);
                    const float cx = fx0 + (float)ox, cy = fy0 + (float)oy, cz = fz0 + (float)oz;
                    const bool fov = cx >= 0 && cx < (float)cd.fW && cy >= 0 && cy < (float)cd.fH;
                    if (!(fov && cz >= 0 && cz < (float)cd.fD)) continue;
                    const int bx = (int)(cx / 8.0f), by = (int)(cy / 8.0f), bz = (int)(cz / 8.0f);
                    const int packed = brick_lookup(*cc, bx, by, bz);
                    if (packed < 0) continue;
                    const int X = ((packed >> 20) & 1023) * 8 + ((int)cx - bx * 8);
                    const int Y = ((packed >> 10) & 1023) * 8 + ((int)cy - by * 8);
                    const int Z = (packed & 1023) * 8 + ((int)cz - bz * 8);
                    if (X < 0 || Y < 0 || Z < 0 || X >= cd.dX * 8 || Y >= cd.dY * 8 || Z >= cd.dZ * 8) continue;
                    const int slot = (X / 8) * cd.dY * cd.dZ + (Y / 8) * cd.dZ + (Z / 8);
                    const size_t vi = (size_t)slot * 512 + (size_t)(Z % 8) * 64 + (Y % 8) * 8 + (X % 8);
                    smp.wsum += w * cc->vox_isset[vi];
                    dsum += w * cc->vox_density[vi];
                    for (int j = 0; j < 8; ++j) lsum[j] += w * lat(vi * 8 + j);
                    smp.vi[smp.nc] = vi;
                    smp.w[smp.nc++] = w;
                }
                for (int j = 0; j < 8; ++j) smp.lat[j] = lsum[j] / smp.wsum;
                forward_head_acts(d, smp.lat, d01, A);
                smp.sigma = std::max(dsum, 1e-6);
            }
            samples.push_back(smp);
            for (int k = 0; k < 3; ++k) rgbv.push_back(sigmoid(A.out[k]));
            if (composite(smp.sigma, A.out, dt, sc->alpha_thre, C, T)) break;
        }
    }
    double loss = 0.0, g[3];
    for (int k = 0; k < 3; ++k) {
        const double e = C[k] + T - (double)target[k];
        loss += e * e * inv_n;
        g[k] = 2.0 * e * inv_n;
    }
    if (pred) { pred[0] = C[0]; pred[1] = C[1]; pred[2] = C[2]; pred[3] = T; }
    if (!(g_table || g_base || g_head || g_lat)) return loss;
    const double gT = g[0] + g[1] + g[2];
    const double x_total = g[0] * C[0] + g[1] * C[1] + g[2] * C[2] + gT * T;
    double Ti = 1.0, x_prefix = 0.0;
    for (size_t i = 0; i < samples.size(); ++i) {
        const S &smp = samples[i];
        const double *c = &rgbv[3 * i];
        double alpha = 1.0 - std::exp(-smp.sigma * (double)smp.dt);
        alpha = std::min(1.0, std::max(0.0, alpha));
        if (!(alpha > (double)sc->alpha_thre)) continue;
        const double gc = g[0] * c[0] + g[1] * c[1] + g[2] * c[2];
        x_prefix += Ti * alpha * gc;
        const double T_next = Ti * (1.0 - alpha);
        const double d_sigma = (double)smp.dt * (T_next * gc - (x_total - x_prefix));
        double d_logit[3];
        for (int k = 0; k < 3; ++k) d_logit[k] = g[k] * Ti * alpha * c[k] * (1.0 - c[k]);
        Acts A;
        if (smp.kind == 0) {
            forward_acts(d, smp.pos, d01, A);
            network_backward(d, smp.pos, A, d_sigma * smp.sigma, d_logit, g_table, g_base, g_head);
        } else {
            forward_head_acts(d, smp.lat, d01, A);
            double din[128];
            head_backward(d, A, d_logit, g_head, din);
            if (g_lat)
                for (int q = 0; q < smp.nc; ++q)
                    for (int j = 0; j < 8; ++j) g_lat[smp.vi[q] * 8 + j] += din[j] * smp.w[q] / smp.wsum;
        }
        Ti = T_next;
        if (Ti < 1e-4) break;
    }
    (void)n;
    return loss;
}

}  // namespace

extern "C" {

/* The cached render's loss and adjoint (see ray_loss_grad_cached), with the
 * voxel latents perturbed by (index into [slots][512][8], delta) pairs. */
double orc_loss_grad_cached(const OrcNet *net, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                            const OrcCache *cc, const OrcCam *ccam, const OrcSteps *cst, const int32_t *pixels, int n_rays,
                            const float *target, double *g_table, double *g_base, double *g_head, double *g_lat,
                            const int64_t *pert_index, const double *pert_delta, int n_pert, int n_threads, double *pred)
{
    NetD d; prepare_net(net, d);
    const LatentSource lat{cc->vox_latents, pert_index, pert_delta, n_pert};
    const double inv_n = 1.0 / (double)std::max(1, n_rays);
    const bool grads = g_table || g_base || g_head || g_lat;
    std::vector<double> per_ray(n_rays, 0.0);
    auto one = [&](int i) {
        const int p = pixels[i];
        per_ray[i] = ray_loss_grad_cached(d, sc, st, cam, bits, cc, ccam, cst, lat, p % cam->W, p / cam->W,
                                          target + 3 * (size_t)i, inv_n, pred ? pred + 4 * (size_t)i : nullptr,
                                          g_table, g_base, g_head, g_lat);
    };
    if (grads) for (int i = 0; i < n_rays; ++i) one(i);
    else parallel_rows(n_rays, n_threads, one);
    double loss = 0.0;
    for (double v : per_ray) loss += v;
    return loss;
}

/* Loss (and, when any gradient pointer is given, its float64 adjoint,
 * accumulated into the given arrays) of the plain render at pixels[i]
 * (y * W + x) against target[3 i .. 3 i + 2].  Perturbations
 * (group 0 table, 1 base blob, 2 head blob; index; delta) are added to the
 * float64 parameters first (finite differences).  pred[4 i] receives
 * (C, T) when non-null.  Gradients run single-threaded (deterministic). */
double orc_loss_grad(const OrcNet *net, const OrcScene *sc, const OrcSteps *st, const OrcCam *cam, const uint8_t *bits,
                     const int32_t *pixels, int n_rays, const float *target, double *g_table, double *g_base, double *g_head,
                     const int32_t *pert_group, const int64_t *pert_index, const double *pert_delta, int n_pert,
                     int n_threads, double *pred)
{
    NetD d; prepare_net(net, d);
    apply_perturbations(d, pert_group, pert_index, pert_delta, n_pert);
    const double inv_n = 1.0 / (double)std::max(1, n_rays);
    const bool grads = g_table || g_base || g_head;
    std::vector<double> per_ray(n_rays, 0.0);
    auto one = [&](int i) {
        const int p = pixels[i];
        per_ray[i] = ray_loss_grad(d, sc, st, cam, bits, p % cam->W, p / cam->W, target + 3 * (size_t)i, inv_n,
                                   pred ? pred + 4 * (size_t)i : nullptr, g_table, g_base, g_head);
    };
    if (grads) for (int i = 0; i < n_rays; ++i) one(i);
    else parallel_rows(n_rays, n_threads, one);
    double loss = 0.0;
    for (double v : per_ray) loss += v;
    return loss;
}

}  /* extern "C" */
