// Intrinsics resample: the 2-D homography warp of the reference's
// camera/homography.py:6-58. Destination pixel (x, y) of batch b samples the
// source image at p = H_b (x, y, 1) after the perspective divide, bilinearly,
// with align_corners semantics (pixel centres at integer coordinates 0..W-1,
// 0..H-1) and zero padding per corner.
//
// Forward: one thread per destination pixel, all channels (the source
// position is shared by the channels). Adjoint: the image gradient scattered
// to the four corners with atomics (caller-zeroed), and the homography
// gradient through the bilinear position derivative and the perspective
// divide, reduced per CTA in a fixed order and per batch element by a second
// kernel (deterministic).
#include <cuda_runtime.h>

#include "../../include/nanodrr_gb300.h"

namespace ndrr {

constexpr int kHomBlock = 256;

struct HomTap {
    float a, b, c;    // H (x, y, 1)
    float sx, sy;     // source position
    int x0, y0;
    float fx, fy;
};

__device__ __forceinline__ HomTap hom_tap(const float* __restrict__ Hm, int x, int y) {
    HomTap t;
    const float fx = (float)x, fy = (float)y;
    t.a = fmaf(__ldg(Hm + 0), fx, fmaf(__ldg(Hm + 1), fy, __ldg(Hm + 2)));
    t.b = fmaf(__ldg(Hm + 3), fx, fmaf(__ldg(Hm + 4), fy, __ldg(Hm + 5)));
    t.c = fmaf(__ldg(Hm + 6), fx, fmaf(__ldg(Hm + 7), fy, __ldg(Hm + 8)));
    t.sx = t.a / t.c;
    t.sy = t.b / t.c;
    // Clamp far-outside positions before the float -> int conversion: beyond
    // one pixel outside the image every corner is zero padding either way.
    const float cx = fminf(fmaxf(t.sx, -2.0f), 1.0e8f), cy = fminf(fmaxf(t.sy, -2.0f), 1.0e8f);
    const float xf = floorf(cx), yf = floorf(cy);
    t.x0 = (int)xf;
    t.y0 = (int)yf;
    t.fx = cx - xf;
    t.fy = cy - yf;
    return t;
}

__global__ void __launch_bounds__(kHomBlock) homography_fwd_kernel(const float* __restrict__ img,
                                                                   const float* __restrict__ hom,
                                                                   float* __restrict__ out, int C, int H, int W) {
    const int b = blockIdx.y;
    const int pix = blockIdx.x * kHomBlock + threadIdx.x;
    if (pix >= H * W) return;
    const int x = pix % W, y = pix / W;
    const HomTap t = hom_tap(hom + (size_t)b * 9, x, y);
    const bool okx0 = t.x0 >= 0 && t.x0 <= W - 1, okx1 = t.x0 + 1 >= 0 && t.x0 + 1 <= W - 1;
    const bool oky0 = t.y0 >= 0 && t.y0 <= H - 1, oky1 = t.y0 + 1 >= 0 && t.y0 + 1 <= H - 1;
    const float w00 = (1.f - t.fx) * (1.f - t.fy), w01 = t.fx * (1.f - t.fy);
    const float w10 = (1.f - t.fx) * t.fy, w11 = t.fx * t.fy;
    const size_t plane = (size_t)H * W;
    for (int c = 0; c < C; ++c) {
        const float* im = img + ((size_t)b * C + c) * plane;
        float v = 0.f;
        if (oky0 && okx0) v = fmaf(w00, __ldg(im + (size_t)t.y0 * W + t.x0), v);
        if (oky0 && okx1) v = fmaf(w01, __ldg(im + (size_t)t.y0 * W + t.x0 + 1), v);
        if (oky1 && okx0) v = fmaf(w10, __ldg(im + (size_t)(t.y0 + 1) * W + t.x0), v);
        if (oky1 && okx1) v = fmaf(w11, __ldg(im + (size_t)(t.y0 + 1) * W + t.x0 + 1), v);
        out[((size_t)b * C + c) * plane + pix] = v;
    }
}

__global__ void __launch_bounds__(kHomBlock) homography_bwd_kernel(const float* __restrict__ go,
                                                                   const float* __restrict__ img,
                                                                   const float* __restrict__ hom,
                                                                   float* __restrict__ gimg,
                                                                   float* __restrict__ partials, int C, int H, int W) {
    __shared__ float red[kHomBlock / 32][9];
    const int b = blockIdx.y;
    const int pix = blockIdx.x * kHomBlock + threadIdx.x;
    float gh[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) gh[j] = 0.f;
    if (pix < H * W) {
        const int x = pix % W, y = pix / W;
        const HomTap t = hom_tap(hom + (size_t)b * 9, x, y);
        const bool okx0 = t.x0 >= 0 && t.x0 <= W - 1, okx1 = t.x0 + 1 >= 0 && t.x0 + 1 <= W - 1;
        const bool oky0 = t.y0 >= 0 && t.y0 <= H - 1, oky1 = t.y0 + 1 >= 0 && t.y0 + 1 <= H - 1;
        const float w00 = (1.f - t.fx) * (1.f - t.fy), w01 = t.fx * (1.f - t.fy);
        const float w10 = (1.f - t.fx) * t.fy, w11 = t.fx * t.fy;
        const size_t plane = (size_t)H * W;
        float dsx = 0.f, dsy = 0.f;
        for (int c = 0; c < C; ++c) {
            const size_t base = ((size_t)b * C + c) * plane;
            const float g = __ldg(go + base + pix);
            if (g == 0.f) continue;
            const float* im = img + base;
            const float v00 = (oky0 && okx0) ? __ldg(im + (size_t)t.y0 * W + t.x0) : 0.f;
            const float v01 = (oky0 && okx1) ? __ldg(im + (size_t)t.y0 * W + t.x0 + 1) : 0.f;
            const float v10 = (oky1 && okx0) ? __ldg(im + (size_t)(t.y0 + 1) * W + t.x0) : 0.f;
            const float v11 = (oky1 && okx1) ? __ldg(im + (size_t)(t.y0 + 1) * W + t.x0 + 1) : 0.f;
            // derivative of the bilinear interpolant in the source position
            dsx = fmaf(g, (1.f - t.fy) * (v01 - v00) + t.fy * (v11 - v10), dsx);
            dsy = fmaf(g, (1.f - t.fx) * (v10 - v00) + t.fx * (v11 - v01), dsy);
            if (gimg != nullptr) {
                float* gi = gimg + base;
                if (oky0 && okx0) atomicAdd(gi + (size_t)t.y0 * W + t.x0, g * w00);
                if (oky0 && okx1) atomicAdd(gi + (size_t)t.y0 * W + t.x0 + 1, g * w01);
                if (oky1 && okx0) atomicAdd(gi + (size_t)(t.y0 + 1) * W + t.x0, g * w10);
                if (oky1 && okx1) atomicAdd(gi + (size_t)(t.y0 + 1) * W + t.x0 + 1, g * w11);
            }
        }
        // Positions clamped above had a zero derivative in the reference too:
        // every corner there is padding, so dsx = dsy = 0 already.
        // sx = a / c, sy = b / c; p = (x, y, 1)
        const float inv_c = 1.f / t.c;
        const float ga = dsx * inv_c, gb = dsy * inv_c;
        const float gc = -(dsx * t.sx + dsy * t.sy) * inv_c;
        const float p[3] = {(float)x, (float)y, 1.f};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            gh[j] = ga * p[j];
            gh[3 + j] = gb * p[j];
            gh[6 + j] = gc * p[j];
        }
    }
    if (partials == nullptr) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        float v = gh[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        float s = 0.f;
        for (int w = 0; w < kHomBlock / 32; ++w) s += red[w][threadIdx.x];
        partials[((size_t)b * gridDim.x + blockIdx.x) * 9 + threadIdx.x] = s;
    }
}

// Per-batch fixed-order sum of the CTA partials into ghom [B, 3, 3].
__global__ void __launch_bounds__(32) homography_reduce_kernel(const float* __restrict__ partials, int nblk,
                                                               float* __restrict__ ghom) {
    const int b = blockIdx.x;
    const int j = threadIdx.x;
    if (j >= 9) return;
    float s = 0.f;
    for (int k = 0; k < nblk; ++k) s += partials[((size_t)b * nblk + k) * 9 + j];
    ghom[(size_t)b * 9 + j] = s;
}

int homography_blocks(int H, int W) { return (H * W + kHomBlock - 1) / kHomBlock; }

cudaError_t launch_homography_fwd(const float* img, const float* hom, int B, int C, int H, int W, float* out,
                                  cudaStream_t st) {
    const dim3 grid((unsigned)homography_blocks(H, W), (unsigned)B);
    homography_fwd_kernel<<<grid, kHomBlock, 0, st>>>(img, hom, out, C, H, W);
    return cudaGetLastError();
}

cudaError_t launch_homography_bwd(const float* go, const float* img, const float* hom, int B, int C, int H, int W,
                                  float* gimg, float* ghom, float* partials, cudaStream_t st) {
    const int nblk = homography_blocks(H, W);
    const dim3 grid((unsigned)nblk, (unsigned)B);
    homography_bwd_kernel<<<grid, kHomBlock, 0, st>>>(go, img, hom, gimg, ghom ? partials : nullptr, C, H, W);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || ghom == nullptr) return e;
    homography_reduce_kernel<<<B, 32, 0, st>>>(partials, nblk, ghom);
    return cudaGetLastError();
}

}  // namespace ndrr
