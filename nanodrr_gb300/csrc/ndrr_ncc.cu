// Normalised cross-correlation of image pairs, forward and adjoint (the
// reference's metrics/ncc.py:8-37 NormalizedCrossCorrelation2d): per plane
// (an image channel, or a patch when the caller unfolds patches into planes)
// both images are centred and scaled by sqrt(population variance + eps), and
// the score of a batch element is the mean over its planes' pixels of the
// product.
//
// Forward: chunks of 4096 pixels per CTA accumulate the raw moments in fp64
// (so centring after the fact keeps full fp32 accuracy), a per-plane kernel
// sums the chunks in a fixed order and forms the centred statistics, and a
// per-batch kernel sums the planes in order. The adjoint is the closed form
// of d score / d x, elementwise from the saved statistics.
#include <cuda_runtime.h>

#include "../../include/nanodrr_gb300.h"

namespace ndrr {

constexpr int kNccBlock = 256;
constexpr int kNccStats = 8;  // mu1, mu2, s1, s2, S12, sum a1, sum a2, plane score
constexpr int kNccChunk = 4096;  // pixels per CTA of the moment pass

static int ncc_chunks(int N) { return (N + kNccChunk - 1) / kNccChunk; }

// Raw moments of one chunk of one plane: sum x1, sum x2, sum x1^2, sum x2^2,
// sum x1 x2 in fp64 (so the centred moments below keep full fp32 accuracy),
// reduced in a fixed order into partials[plane][chunk][5].
__global__ void __launch_bounds__(kNccBlock) ncc_moments_kernel(const float* __restrict__ x1,
                                                                const float* __restrict__ x2, int N,
                                                                double* __restrict__ partials) {
    __shared__ double sh[kNccBlock / 32][5];
    const size_t plane = blockIdx.x;
    const int chunk = blockIdx.y, nch = gridDim.y;
    const int beg = chunk * kNccChunk, end = min(N, beg + kNccChunk);
    const float* a = x1 + plane * N;
    const float* b = x2 + plane * N;
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = beg + threadIdx.x; i < end; i += kNccBlock) {
        const double u = (double)__ldg(a + i), v = (double)__ldg(b + i);
        s[0] += u;
        s[1] += v;
        s[2] = fma(u, u, s[2]);
        s[3] = fma(v, v, s[3]);
        s[4] = fma(u, v, s[4]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        double x = s[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[warp][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double x = 0.0;
        for (int w = 0; w < kNccBlock / 32; ++w) x += sh[w][threadIdx.x];
        partials[(plane * nch + chunk) * 5 + threadIdx.x] = x;
    }
}

// Per plane: fixed-order sum of the chunk moments, then the centred
// statistics and the plane's score.
__global__ void __launch_bounds__(32) ncc_stats_kernel(const double* __restrict__ partials, int nch, int N,
                                                       float eps, float* __restrict__ stats, int planes) {
    const int plane = blockIdx.x * 32 + threadIdx.x;
    if (plane >= planes) return;
    double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < nch; ++c)
        for (int k = 0; k < 5; ++k) m[k] += partials[((size_t)plane * nch + c) * 5 + k];
    const double n = (double)N;
    const double mu1 = m[0] / n, mu2 = m[1] / n;
    const double c11 = fmax(m[2] - n * mu1 * mu1, 0.0), c22 = fmax(m[3] - n * mu2 * mu2, 0.0);
    const double c12 = m[4] - n * mu1 * mu2;
    const double s1 = sqrt(c11 / n + (double)eps), s2 = sqrt(c22 / n + (double)eps);
    float* st = stats + (size_t)plane * kNccStats;
    st[0] = (float)mu1;
    st[1] = (float)mu2;
    st[2] = (float)s1;
    st[3] = (float)s2;
    st[4] = (float)c12;
    st[5] = (float)(m[0] - n * mu1);  // centred first moments: zero up to rounding
    st[6] = (float)(m[1] - n * mu2);
    st[7] = (float)(c12 / (s1 * s2));
}

__global__ void __launch_bounds__(32) ncc_score_kernel(const float* __restrict__ stats, int P, int N,
                                                       float* __restrict__ score, int B) {
    const int b = blockIdx.x * 32 + threadIdx.x;
    if (b >= B) return;
    double s = 0.0;
    for (int p = 0; p < P; ++p) s += (double)stats[((size_t)b * P + p) * kNccStats + 7];
    score[b] = (float)(s / ((double)P * N));
}

// d score_b / d x1_j = g [ x2n_j / s1 - sum(x2n) / (N s1) - a1_j S12 / (s2 N s1^3) ],
// g = go_b / (P N), x2n = (x2 - mu2) / s2; symmetric for x2.
__global__ void __launch_bounds__(kNccBlock) ncc_bwd_kernel(const float* __restrict__ go,
                                                            const float* __restrict__ x1,
                                                            const float* __restrict__ x2,
                                                            const float* __restrict__ stats, int P, int N,
                                                            float* __restrict__ g1, float* __restrict__ g2) {
    const size_t plane = blockIdx.x;
    const int b = (int)(plane / P);
    const float* st = stats + plane * kNccStats;
    const float m1 = st[0], m2 = st[1], s1 = st[2], s2 = st[3], S12 = st[4], z1 = st[5], z2 = st[6];
    const float g = __ldg(go + b) / ((float)P * (float)N);
    const float inv_n = 1.f / (float)N;
    // x1 side
    const float k1a = g / (s1 * s2), k1b = g * z2 / (s2 * N * s1), k1c = g * S12 * inv_n / (s2 * s1 * s1 * s1);
    const float k2a = g / (s1 * s2), k2b = g * z1 / (s1 * N * s2), k2c = g * S12 * inv_n / (s1 * s2 * s2 * s2);
    const float* a = x1 + plane * N;
    const float* c = x2 + plane * N;
    const int beg = blockIdx.y * kNccChunk, end = min(N, beg + kNccChunk);
    for (int i = beg + threadIdx.x; i < end; i += kNccBlock) {
        const float d1 = __ldg(a + i) - m1, d2 = __ldg(c + i) - m2;
        if (g1 != nullptr) g1[plane * N + i] = k1a * d2 - k1b - k1c * d1;
        if (g2 != nullptr) g2[plane * N + i] = k2a * d1 - k2b - k2c * d2;
    }
}

size_t ncc_workspace_bytes(int B, int P, int N) { return (size_t)B * P * ncc_chunks(N) * 5 * sizeof(double); }

cudaError_t launch_ncc_fwd(const float* x1, const float* x2, int B, int P, int N, float eps, float* score,
                           float* stats, void* workspace, cudaStream_t st) {
    const int planes = B * P, nch = ncc_chunks(N);
    double* partials = reinterpret_cast<double*>(workspace);
    ncc_moments_kernel<<<dim3((unsigned)planes, (unsigned)nch), kNccBlock, 0, st>>>(x1, x2, N, partials);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    ncc_stats_kernel<<<(planes + 31) / 32, 32, 0, st>>>(partials, nch, N, eps, stats, planes);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ncc_score_kernel<<<(B + 31) / 32, 32, 0, st>>>(stats, P, N, score, B);
    return cudaGetLastError();
}

cudaError_t launch_ncc_bwd(const float* go, const float* x1, const float* x2, const float* stats, int B, int P,
                           int N, float* g1, float* g2, cudaStream_t st) {
    ncc_bwd_kernel<<<dim3((unsigned)((size_t)B * P), (unsigned)ncc_chunks(N)), kNccBlock, 0, st>>>(go, x1, x2, stats,
                                                                                                 P, N, g1, g2);
    return cudaGetLastError();
}

}  // namespace ndrr
