// Camera-space ray endpoints of a detector in one launch: the reference's
// _make_tgt / _make_src (src/nanodrr/drr/renderer.py:101-132), which as
// tensor expressions take a dozen small launches per render call.
//
// tgt[b, n] = sdd[b] * (K0 * (u + 0.5) + K1 * (v + 0.5) + K2), n = v * W + u,
// where Kc is column c of K^-1[b]; every product and sum is rounded on its
// own and summed left to right, the order of the broadcast expression
// (renderer.py::_make_tgt), so the rays are bitwise those of the tensor path.
// src is the camera origin ([B, 1, 3] zeros) for a pinhole, or tgt with
// z - sdd ([B, N, 3]) for parallel rays.
#include <cuda_runtime.h>

#include "ndrr_launch.h"

namespace ndrr {

__global__ void __launch_bounds__(256) camera_rays_kernel(const float* __restrict__ k_inv, int k_stride,
                                                          const float* __restrict__ sdd, int s_stride, int B,
                                                          int height, int width, int orthographic,
                                                          float* __restrict__ src, float* __restrict__ tgt) {
    const long long N = (long long)height * width;
    const long long total = (long long)B * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(i / N);
        const long long n = i - (long long)b * N;
        const int v = (int)(n / width), u = (int)(n - (long long)v * width);
        const float uf = __fadd_rn((float)u, 0.5f), vf = __fadd_rn((float)v, 0.5f);
        const float* k = k_inv + (long long)b * k_stride;
        const float s = sdd[(long long)b * s_stride];
        float t[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            // K[r,2] * 1 is exact, so the third term adds K[r,2] itself.
            const float ray = __fadd_rn(__fadd_rn(__fmul_rn(k[3 * r + 0], uf), __fmul_rn(k[3 * r + 1], vf)), k[3 * r + 2]);
            t[r] = __fmul_rn(s, ray);
        }
        float* o = tgt + 3 * i;
        o[0] = t[0];
        o[1] = t[1];
        o[2] = t[2];
        if (orthographic) {
            float* p = src + 3 * i;
            p[0] = t[0];
            p[1] = t[1];
            p[2] = __fsub_rn(t[2], s);
        } else if (n == 0) {
            float* p = src + 3 * (long long)b;
            p[0] = 0.f;
            p[1] = 0.f;
            p[2] = 0.f;
        }
    }
}

cudaError_t launch_camera_rays(const float* k_inv, int n_k, const float* sdd, int n_s, int B, int height, int width,
                               int orthographic, float* src, float* tgt, cudaStream_t st) {
    const long long total = (long long)B * height * width;
    const long long blocks = (total + 255) / 256;
    const int grid = (int)(blocks < 152 * 16 ? blocks : 152 * 16);
    camera_rays_kernel<<<grid, 256, 0, st>>>(k_inv, n_k == 1 ? 0 : 9, sdd, n_s == 1 ? 0 : 1, B, height, width,
                                             orthographic, src, tgt);
    return cudaGetLastError();
}

}  // namespace ndrr
