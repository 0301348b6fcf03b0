/*
 * ref_composite.cu - runs the reference's own compositing kernel on the host
 * to make golden vectors.  TEST INFRASTRUCTURE ONLY (built by oracle/Makefile
 * into oracle/_ref/, never part of the product).
 *
 * The kernel is accumulate_performance_kernel (src/performance_renderer.cu:
 * 71-125).  Its text is taken unchanged from the reference tree at build time
 * (the Makefile cuts it out of the file into oracle/_ref/, which is not
 * committed) and compiled here by nvcc as a host function: __global__ becomes
 * static and threadIdx / blockIdx / blockDim are host variables, so one call
 * with threadIdx.x = ray runs the kernel's thread for that ray.  The
 * reference headers (include/common.h, include/raymarch_common.h,
 * include/renderer_common.h) come unchanged through -I.  Host arithmetic
 * (libm expf, IEEE division) stands in for the device's.
 *
 * Input (binary, little endian, written by tests/golden/make_golden_composite.py):
 *   int32 n_alive, batch_size; float cone_angle, dt_min, dt_max, alpha_thre;
 *   int32 n_steps[n_alive]; uint8 alive[n_alive]; float result[4 * n_alive] (rgb, T);
 *   uint16 network_output[4 * batch_size] (fp16 bits: rows r, g, b, log-density, each batch_size long);
 *   float t0[batch_size]
 *   (the sample-major layout of the kernel: sample s of ray i is row s * n_alive + i)
 * Output: float result[4 * n_alive]; uint8 alive[n_alive].
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "raymarch_common.h"
#include "renderer_common.h"

static uint3 g_thread_idx, g_block_idx;
static dim3 g_block_dim;
#undef __global__
#define __global__ static
#define threadIdx g_thread_idx
#define blockIdx g_block_idx
#define blockDim g_block_dim
#include "composite_kernel.inc"
#undef threadIdx
#undef blockIdx
#undef blockDim
#undef __global__

template <class T> static void rd(FILE *f, T *p, size_t n = 1)
{
    if (fread(p, sizeof(T), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
template <class T> static void wr(FILE *f, const T *p, size_t n = 1) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char **argv)
{
    if (argc != 3) { fprintf(stderr, "usage: ref_composite in.bin out.bin\n"); return 1; }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 1;
    int n_alive = 0, batch = 0;
    float cone = 0, dt_min = 0, dt_max = 0, thre = 0;
    rd(f, &n_alive); rd(f, &batch);
    rd(f, &cone); rd(f, &dt_min); rd(f, &dt_max); rd(f, &thre);
    std::vector<int> n_steps(n_alive);
    std::vector<unsigned char> alive8(n_alive);
    std::vector<float> res(4 * (size_t)n_alive), t0(batch);
    std::vector<unsigned short> out16(4 * (size_t)batch);
    rd(f, n_steps.data(), n_alive);
    rd(f, alive8.data(), n_alive);
    rd(f, res.data(), res.size());
    rd(f, out16.data(), out16.size());
    rd(f, t0.data(), t0.size());
    fclose(f);

    RaymarchInfo rm{};
    rm.stepsize_info.cone_angle = cone;
    rm.stepsize_info.dt_min = dt_min;
    rm.stepsize_info.dt_max = dt_max;
    SceneInfo sc{};
    sc.alpha_thre = thre;
    std::vector<BaseRayResult> results(n_alive);
    std::vector<int> alive(n_alive);
    for (int i = 0; i < n_alive; ++i) {
        results[i].rgb = make_float3(res[4 * i], res[4 * i + 1], res[4 * i + 2]);
        results[i].transmittance = res[4 * i + 3];
        alive[i] = alive8[i];
    }
    std::vector<half> outh(out16.size());
    for (size_t k = 0; k < out16.size(); ++k) outh[k] = __ushort_as_half(out16[k]);

    g_block_idx = make_uint3(0, 0, 0);
    g_block_dim = dim3((unsigned)n_alive, 1, 1);
    for (int i = 0; i < n_alive; ++i) {
        g_thread_idx = make_uint3((unsigned)i, 0, 0);
        accumulate_performance_kernel(n_alive, batch, rm, sc, results.data(), n_steps.data(), alive.data(), outh.data(), t0.data());
    }

    FILE *o = fopen(argv[2], "wb");
    if (!o) return 1;
    for (int i = 0; i < n_alive; ++i) {
        const float v[4] = {results[i].rgb.x, results[i].rgb.y, results[i].rgb.z, results[i].transmittance};
        wr(o, v, 4);
    }
    for (int i = 0; i < n_alive; ++i) {
        const unsigned char a = alive[i] ? 1 : 0;
        wr(o, &a);
    }
    fclose(o);
    return 0;
}
