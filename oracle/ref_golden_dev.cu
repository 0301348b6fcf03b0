/*
 * ref_golden_dev.cu - the reference's marcher math compiled for the GPU with
 * the reference's own device flags, to make device golden vectors.  TEST
 * INFRASTRUCTURE ONLY (built by oracle/Makefile into oracle/_ref/, never part
 * of the product).
 *
 * The reference builds its kernels with -use_fast_math (CMakeLists.txt:13):
 * approximate division and square root, __logf/__expf for logf/expf and
 * flush-to-zero, with nvcc's default fused multiply-add contraction.  Its
 * host-side golden vectors (ref_golden.cu) therefore pin the host arithmetic
 * only.  This file includes the same reference headers unchanged and runs
 * their device code, one thread per pixel, in the order of the reference's
 * two device kernels for the plain path:
 *   initRayPayloads_split_kernel   src/renderer.cu:86-131 (deterministic pixel
 *                                  centre, generateRay, ray_aabb_intersect,
 *                                  valid_t_from_t, far = min(t1, far))
 *   sample_performance_kernel      src/performance_renderer.cu:15-70 (t1 = t0 +
 *                                  calculate_stepsize(t0), stop when the
 *                                  midpoint passes far, grid_occupied_at<128,
 *                                  true> at origin + t_mid * dir)
 * over all steps of the ray (the sub-iteration split does not change them).
 *
 * The RaymarchInfo and SceneInfo come as raw structs written by ref_golden
 * (host side, where StepsizeInfo::setAdditionalInfo runs in the reference
 * too).  Output per pixel (int32 x4): hits, steps, occupied steps, FNV-1a
 * hash of the occupied steps' t0 bit patterns.  The kernel is launched by
 * tests/golden/make_golden_dev.py through the CUDA driver API.
 *
 * Bounds: every read of grid_bitfield is at byte (mip * 128^3 + morton) / 8
 * with mip < grid_nlvl and morton < 8 * 128^3 (a coordinate rounded up to
 * 128 sets bit 21 of the Morton code at most once per axis), so the launcher
 * allocates (grid_nlvl + 7) * 128^3 / 8 bytes, zero beyond the grid.
 */
#include <cuda_runtime.h>
#include <cstdint>

#include "raymarch_common.h"

extern "C" __global__ void golden_march_dev(const RaymarchInfo *__restrict__ rm_p, const SceneInfo *__restrict__ si_p,
                                            const uint8_t *__restrict__ bits, const int *__restrict__ pix, int n_pix,
                                            int max_steps, int *__restrict__ out)
{
    const int i = threadIdx.x + blockIdx.x * blockDim.x;
    if (i >= n_pix)
        return;
    const RaymarchInfo rm_info = *rm_p;
    const SceneInfo scene_info = *si_p;
    const int x = pix[2 * i], y = pix[2 * i + 1];
    const int ray_id = y * rm_info.cam_info.resolution.x + x;
    const float2 screen_point = make_float2(x + 0.5f, y + 0.5f);
    const FrustumRay ray = generateRay(ray_id, screen_point, rm_info);
    float aabb_t0, aabb_t1;
    const bool hits = ray_aabb_intersect(ray, scene_info.aabb_from, scene_info.aabb_to, aabb_t0, aabb_t1);
    const float far_ = hits ? min(aabb_t1, rm_info.stepsize_info.far) : rm_info.stepsize_info.far;
    const float start_t = hits ? valid_t_from_t(aabb_t0, rm_info.stepsize_info) : rm_info.stepsize_info.near;
    const float start_dt = calculate_stepsize(start_t, rm_info.stepsize_info);
    float t1 = start_t + start_dt * 0.0f;
    int steps = 0, occupied = 0;
    uint32_t h = 2166136261u;
    if (hits) {
        while (steps < max_steps) {
            const float t0 = t1;
            const float dt = calculate_stepsize(t0, rm_info.stepsize_info);
            t1 = t0 + dt;
            const float t_mid = (t0 + t1) * 0.5f;
            if (t_mid > far_)
                break;
            ++steps;
            const float3 world_point = ray.origin + t_mid * ray.dir;
            if (grid_occupied_at<128, true>(world_point, scene_info, bits)) {
                ++occupied;
                uint32_t b = __float_as_uint(t0);
                for (int k = 0; k < 4; ++k, b >>= 8)
                    h = (h ^ (b & 255u)) * 16777619u;
            }
        }
    }
    out[4 * i + 0] = hits;
    out[4 * i + 1] = steps;
    out[4 * i + 2] = occupied;
    out[4 * i + 3] = (int)h;
}
