/*
 * ref_golden.cu - runs the reference's own marcher math on the host to make
 * golden vectors.  TEST INFRASTRUCTURE ONLY (built by oracle/Makefile into
 * oracle/_ref/, never part of the product).
 *
 * It includes the reference headers unchanged (include/raymarch_common.h,
 * include/common.h from the reference tree, passed with -I) and drives them
 * exactly as the reference kernels do:
 *   StepsizeInfo::setAdditionalInfo          include/common.h:109-131
 *   generateRay (deterministic pixel centre)  include/raymarch_common.h:218-251
 *   ray_aabb_intersect / valid_t_from_t       :482-532, :286-296
 *   sample_performance_kernel step loop       src/performance_renderer.cu:39-62
 *   grid_occupied_at<128, true>               include/raymarch_common.h:680-710
 *   apply_contraction, cam2froxel             :610-653, :316-336
 * The Morton bitfield is made from the uint8 grid with the reference's own
 * morton3D_invert, as occupancy_grid_to_morton_kernel does (src/loader.cu:20-55).
 *
 * Input (binary, little endian, written by tests/golden/make_golden.py):
 *   int32 nlvl, contraction; float aabb[6], caabb[6]; float cone, stepsize, near, far;
 *   int32 W, H; float fx, fy, px, py; float c2w[12];
 *   int32 n_pix; int32 pix[2*n_pix]; int32 max_steps;
 *   int32 n_pts; float pts[3*n_pts];
 *   uint8 grid[nlvl*128^3]
 * Output: see write_out below.  With a third argument it also writes the
 * input of the device march (ref_golden_dev.cu): sizeof(RaymarchInfo),
 * sizeof(SceneInfo), both structs' bytes, the pixel list, max_steps, nlvl and
 * the Morton bitfield.
 */
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "raymarch_common.h"

template <class T> static void rd(FILE *f, T *p, size_t n = 1)
{
    if (fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
template <class T> static void wr(FILE *f, const T *p, size_t n = 1) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char **argv)
{
    if (argc != 3 && argc != 4) { fprintf(stderr, "usage: ref_golden in.bin out.bin [device_input.bin]\n"); return 1; }
    FILE *fi = fopen(argv[1], "rb");
    if (!fi) return 1;
    int nlvl, contraction;
    float aabb[6], caabb[6], cone, stepsize, nearv, farv;
    rd(fi, &nlvl); rd(fi, &contraction); rd(fi, aabb, 6); rd(fi, caabb, 6);
    rd(fi, &cone); rd(fi, &stepsize); rd(fi, &nearv); rd(fi, &farv);
    int W, H; float fx, fy, px, py, c2w[12];
    rd(fi, &W); rd(fi, &H); rd(fi, &fx); rd(fi, &fy); rd(fi, &px); rd(fi, &py); rd(fi, c2w, 12);
    int n_pix; rd(fi, &n_pix);
    std::vector<int> pix(2 * (size_t)n_pix); rd(fi, pix.data(), pix.size());
    int max_steps; rd(fi, &max_steps);
    int n_pts; rd(fi, &n_pts);
    std::vector<float> pts(3 * (size_t)n_pts); rd(fi, pts.data(), pts.size());
    const int R = 128, vals = R * R * R;
    std::vector<uint8_t> grid((size_t)vals * nlvl); rd(fi, grid.data(), grid.size());
    fclose(fi);

    SceneInfo si{};
    si.grid_resolution = R; si.grid_nlvl = nlvl; si.vals_per_lvl = vals; si.normalized = false;
    si.aabb_from = make_float3(aabb[0], aabb[1], aabb[2]); si.aabb_to = make_float3(aabb[3], aabb[4], aabb[5]);
    si.contraction_aabb_from = make_float3(caabb[0], caabb[1], caabb[2]);
    si.contraction_aabb_to = make_float3(caabb[3], caabb[4], caabb[5]);
    si.contraction_type = contraction ? WARP_AABB_LINF : AABB;
    si.is_open_gl = false; si.alpha_thre = 0.0f;
    StepsizeInfo st{};
    st.cone_angle = cone; st.stepsize = stepsize; st.near = nearv; st.far = farv;
    st.setAdditionalInfo(si);

    CameraInfo ci{};
    ci.resolution = make_int2(W, H); ci.is_open_gl = false;
    ci.focal = make_float2(fx, fy); ci.principal = make_float2(px, py);
    ci.cam2world = {make_float4(c2w[0], c2w[1], c2w[2], c2w[3]), make_float4(c2w[4], c2w[5], c2w[6], c2w[7]),
                    make_float4(c2w[8], c2w[9], c2w[10], c2w[11])};
    ci.world2cam = ci.cam2world.inverse();
    RaymarchInfo rm{};
    rm.cam_info = ci; rm.next_cam_info = ci; rm.stepsize_info = st;
    rm.sample_index = 0; rm.motion_blur = false; rm.deterministic = true;

    std::vector<uint8_t> bits((size_t)vals * nlvl / 8, 0);
    for (int i = 0; i < vals * nlvl; ++i) {
        const int lvl = i / vals, j = i % vals;
        const uint32_t x = morton3D_invert(j >> 0), y = morton3D_invert(j >> 1), z = morton3D_invert(j >> 2);
        if (grid[(size_t)lvl * vals + x * R * R + y * R + z]) bits[i / 8] |= (uint8_t)(1u << (i % 8));
    }

    if (argc == 4) {
        /* input of ref_golden_dev.cu's device march: the structs as the reference's host hands them
         * to its kernels, the Morton bitfield and the pixel list */
        FILE *fd = fopen(argv[3], "wb");
        if (!fd) return 1;
        const int srm = (int)sizeof(RaymarchInfo), ssi = (int)sizeof(SceneInfo), nb = (int)bits.size();
        wr(fd, &srm); wr(fd, &ssi); wr(fd, &rm); wr(fd, &si);
        wr(fd, &n_pix); wr(fd, pix.data(), pix.size()); wr(fd, &max_steps);
        wr(fd, &nlvl); wr(fd, &nb); wr(fd, bits.data(), bits.size());
        fclose(fd);
    }

    FILE *fo = fopen(argv[2], "wb");
    if (!fo) return 1;
    /* derived step info */
    wr(fo, &st.dt_min); wr(fo, &st.dt_max); wr(fo, &st.t_min); wr(fo, &st.t_max);
    wr(fo, &st.i_min); wr(fo, &st.i_max); wr(fo, &st.log1p_c); wr(fo, &st.near_i);
    const CameraMatrix inv = ci.world2cam;
    wr(fo, &inv, 1);
    const float max_step = max_step_in_scene(st, si);
    wr(fo, &max_step);
    /* per pixel: hits, start, far, n_steps, then per step t0 and occupancy */
    for (int p = 0; p < n_pix; ++p) {
        const int x = pix[2 * p], y = pix[2 * p + 1];
        const float2 sp = make_float2(x + 0.5f, y + 0.5f);
        const FrustumRay ray = generateRay(y * W + x, sp, rm);
        float t0a, t1a;
        const bool hits = ray_aabb_intersect(ray, si.aabb_from, si.aabb_to, t0a, t1a);
        const float far_ = hits ? min(t1a, st.far) : st.far;
        const float start = hits ? valid_t_from_t(t0a, st) : st.near;
        std::vector<float> t0s; std::vector<uint8_t> occ;
        float t1 = start + 0.0f;
        if (hits) {
            for (int s = 0; s < max_steps; ++s) {
                const float t0 = t1;
                const float dt = calculate_stepsize(t0, st);
                t1 = t0 + dt;
                const float tm = (t0 + t1) * 0.5f;
                if (tm > far_) break;
                const float3 wp = ray.origin + tm * ray.dir;
                t0s.push_back(t0);
                occ.push_back(grid_occupied_at<128, true>(wp, si, bits.data()) ? 1 : 0);
            }
        }
        const int hi = hits, n = (int)t0s.size();
        wr(fo, &hi); wr(fo, &start); wr(fo, &far_); wr(fo, &ray.origin); wr(fo, &ray.dir); wr(fo, &n);
        wr(fo, t0s.data(), t0s.size()); wr(fo, occ.data(), occ.size());
    }
    /* per point: step_from_t(|p|), t_from_step(|p|*100), contraction, occupancy, cam2froxel */
    for (int i = 0; i < n_pts; ++i) {
        const float3 p = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        const float a = fabsf(p.x) * 4.0f + 0.001f;
        const float sft = st.step_from_t(a);
        const float tfs = st.t_from_step(a * 100.0f);
        const float3 c = apply_contraction(p, si);
        const int o = grid_occupied_at<128, true>(p, si, bits.data()) ? 1 : 0;
        float tf;
        const float3 fr = world2froxel(p, ci, st, tf);
        wr(fo, &sft); wr(fo, &tfs); wr(fo, &c); wr(fo, &o); wr(fo, &fr); wr(fo, &tf);
    }
    /* integer helpers */
    for (int i = 0; i < 64; ++i) {
        const uint32_t m = morton3D(i * 7 % 128, i * 13 % 128, i * 29 % 128);
        const int pk = pack3D(make_int3(i * 3 % 1024, i * 5 % 1024, i * 11 % 1024));
        const int3 t3 = to3D(i * 977, make_int3(128, 128, 16));
        wr(fo, &m); wr(fo, &pk); wr(fo, &t3);
    }
    fclose(fo);
    return 0;
}
