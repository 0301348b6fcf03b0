/*
 * ref_sampling.cu - runs the reference's own sampling code of
 * non-deterministic ray generation on the host to make golden vectors.
 * TEST INFRASTRUCTURE ONLY (built by oracle/Makefile into oracle/_ref/, never
 * part of the product).
 *
 * It includes the reference headers unchanged (include/raymarch_common.h,
 * which brings include/util/random_val.h and include/util/quat.h) and calls:
 *   sobol, ld_random_val              include/util/random_val.h:166-290
 *   ld_random_pixel_offset / _t_offset :320-331
 *   square2disk_shirley               :108-127
 *   camera_slerp                      include/raymarch_common.h:208-216
 *   generateRay (deterministic = false, depth of field, motion blur)
 *                                     include/raymarch_common.h:218-251
 *   with the start t of initRayPayloads_split_kernel (src/renderer.cu:99-124)
 *
 * Input (binary, little endian, written by tests/golden/make_golden_sampling.py):
 *   int32 n_sobol; uint32 (index, dim)[n_sobol]
 *   int32 n_ld; uint32 (index, seed)[n_ld]
 *   int32 n_spp; uint32 spp[n_spp]
 *   int32 n_t; uint32 (spp, ray_id)[n_t]
 *   int32 n_disk; float (a, b)[n_disk]
 *   int32 n_slerp; float (a[12], b[12], t)[n_slerp]
 *   camera: int32 W, H; float fx, fy, px, py, c2w[12], nc2w[12], aperature, focus_z;
 *   scene/steps: float aabb[6], cone, stepsize, near, far; int32 nlvl
 *   int32 n_rays; int32 (px, py, spp, flags)[n_rays]   flags: 1 motion blur, 2 depth of field
 * Output: the values in the same order (see tests/golden/make_golden_sampling.py).
 */
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "raymarch_common.h"

template <class T> static void rd(FILE *f, T *p, size_t n = 1)
{
    if (fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
template <class T> static void wr(FILE *f, const T *p, size_t n = 1) { fwrite(p, sizeof(T), n, f); }

static CameraMatrix mat(const float *m)
{
    CameraMatrix c;
    c.m0 = make_float4(m[0], m[1], m[2], m[3]);
    c.m1 = make_float4(m[4], m[5], m[6], m[7]);
    c.m2 = make_float4(m[8], m[9], m[10], m[11]);
    return c;
}

int main(int argc, char **argv)
{
    if (argc != 3) { fprintf(stderr, "usage: ref_sampling in.bin out.bin\n"); return 1; }
    FILE *fi = fopen(argv[1], "rb"), *fo = fopen(argv[2], "wb");
    if (!fi || !fo) return 1;
    int n;
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        uint32_t idx, dim; rd(fi, &idx); rd(fi, &dim);
        const uint32_t v = sobol(idx, dim); wr(fo, &v);
    }
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        uint32_t idx, seed; rd(fi, &idx); rd(fi, &seed);
        const float v = ld_random_val(idx, seed); wr(fo, &v);
        const float2 v2 = ld_random_val_2d(idx, seed); wr(fo, &v2);
    }
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        uint32_t spp; rd(fi, &spp);
        const float2 o = ld_random_pixel_offset(spp); wr(fo, &o);
    }
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        uint32_t spp, ray; rd(fi, &spp); rd(fi, &ray);
        const float o = ld_random_t_offset(spp, ray * 56924617u); wr(fo, &o);
    }
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        float a, b; rd(fi, &a); rd(fi, &b);
        const float2 d = square2disk_shirley(make_float2(a, b)); wr(fo, &d);
    }
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        float a[12], b[12], t; rd(fi, a, 12); rd(fi, b, 12); rd(fi, &t);
        const CameraMatrix m = camera_slerp(mat(a), mat(b), t);
        wr(fo, &m);
    }
    int W, H; float fx, fy, px, py, c2w[12], nc2w[12], aper, focus;
    rd(fi, &W); rd(fi, &H); rd(fi, &fx); rd(fi, &fy); rd(fi, &px); rd(fi, &py); rd(fi, c2w, 12); rd(fi, nc2w, 12);
    rd(fi, &aper); rd(fi, &focus);
    float aabb[6], cone, stepsize, nearv, farv; int nlvl;
    rd(fi, aabb, 6); rd(fi, &cone); rd(fi, &stepsize); rd(fi, &nearv); rd(fi, &farv); rd(fi, &nlvl);
    SceneInfo si{};
    si.grid_resolution = 128; si.grid_nlvl = nlvl; si.vals_per_lvl = 128 * 128 * 128; si.normalized = false;
    si.aabb_from = make_float3(aabb[0], aabb[1], aabb[2]); si.aabb_to = make_float3(aabb[3], aabb[4], aabb[5]);
    si.contraction_aabb_from = si.aabb_from; si.contraction_aabb_to = si.aabb_to;
    si.contraction_type = AABB; si.is_open_gl = false; si.alpha_thre = 0.0f;
    StepsizeInfo st{};
    st.cone_angle = cone; st.stepsize = stepsize; st.near = nearv; st.far = farv;
    st.setAdditionalInfo(si);
    rd(fi, &n);
    for (int i = 0; i < n; ++i) {
        int q[4]; rd(fi, q, 4);
        CameraInfo ci{};
        ci.resolution = make_int2(W, H); ci.is_open_gl = false;
        ci.focal = make_float2(fx, fy); ci.principal = make_float2(px, py);
        ci.cam2world = mat(c2w); ci.world2cam = ci.cam2world.inverse();
        ci.aperature = (q[3] & 2) ? aper : 0.0f; ci.focus_z = focus;
        CameraInfo cn = ci;
        cn.cam2world = mat(nc2w); cn.world2cam = cn.cam2world.inverse();
        RaymarchInfo rm{};
        rm.cam_info = ci; rm.next_cam_info = cn; rm.stepsize_info = st;
        rm.sample_index = q[2]; rm.motion_blur = (q[3] & 1) != 0; rm.deterministic = false;
        /* initRayPayloads_split_kernel, src/renderer.cu:99-124 */
        const int ray_id = q[1] * W + q[0];
        const float2 off = ld_random_pixel_offset(rm.sample_index);
        const float2 sp = make_float2(q[0] + off.x, q[1] + off.y);
        const FrustumRay ray = generateRay(ray_id, sp, rm);
        float t0, t1;
        const bool hits = ray_aabb_intersect(ray, si.aabb_from, si.aabb_to, t0, t1);
        const float start_t = hits ? valid_t_from_t(t0, st) : st.near;
        const float start_dt = calculate_stepsize(start_t, st);
        const float t_off = start_dt * ld_random_t_offset(rm.sample_index, ray_id * 56924617);
        const float v[8] = {ray.origin.x, ray.origin.y, ray.origin.z, ray.dir.x, ray.dir.y, ray.dir.z,
                            hits ? start_t + t_off : 0.0f, hits ? 1.0f : 0.0f};
        wr(fo, v, 8);
    }
    fclose(fi);
    fclose(fo);
    return 0;
}
