// Training and packing kernels of the learned empty-space proposal network
// (architecture and feature encoding in ndrr_proposal.cuh). Training runs in
// fp32 on the CUDA cores: a fused kernel evaluates the network on a chunk of
// rays, the asymmetric loss, the backward pass and the weight gradients
// (reduced in registers per CTA, one atomic per parameter per CTA); Adam
// updates the fp32 master parameters; `pack` converts them to the bf16
// layout the render kernels' tensor-core inference reads.
#include <algorithm>
#include <cstdio>

#include "ndrr_device.cuh"
#include "ndrr_launch.h"
#include "ndrr_proposal.cuh"

namespace ndrr {

// ------------------------------------------------------------------ dataset
// Features and targets for every ray of a batch of poses. Targets are the
// fractions (f_near, f_far) of the in-box segment where the plain march saw
// its first and last non-empty sample (`extent`, in t), widened on each side
// by `widen` voxels of Chebyshev distance along the ray (the resolution at
// which the occupancy grid can confirm emptiness: cell size plus dilation);
// rays without a non-empty sample get the empty interval (1, 0). Rays whose
// line misses the footprint box are marked invalid.
__global__ void proposal_dataset_kernel(const float* __restrict__ M, const float* __restrict__ src,
                                        const float* __restrict__ tgt, int src_per_ray, int B, int N, int D, int H,
                                        int W, const float* __restrict__ extent, float widen, float* __restrict__ X,
                                        float* __restrict__ T, uint8_t* __restrict__ valid) {
    const long long total = (long long)B * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(i / N);
        const float* m = M + (size_t)b * 12;
        const float* sp = src_per_ray ? src + i * 3 : src + (size_t)b * 3;
        const float sx = sp[0], sy = sp[1], sz = sp[2];
        const float ex = tgt[i * 3 + 0] - sx, ey = tgt[i * 3 + 1] - sy, ez = tgt[i * 3 + 2] - sz;
        Ray r;
        r.p0x = m[0] * sx + m[1] * sy + m[2] * sz + m[3];
        r.p0y = m[4] * sx + m[5] * sy + m[6] * sz + m[7];
        r.p0z = m[8] * sx + m[9] * sy + m[10] * sz + m[11];
        r.dx = m[0] * ex + m[1] * ey + m[2] * ez;
        r.dy = m[4] * ex + m[5] * ey + m[6] * ez;
        r.dz = m[8] * ex + m[9] * ey + m[10] * ez;
        float tau0, tau1, f[kPropIn];
        const bool hit = proposal_features(r, D, H, W, tau0, tau1, f);
        for (int k = 0; k < kPropIn; ++k) X[i * kPropIn + k] = f[k];
        const float e0 = extent[i * 2], e1 = extent[i * 2 + 1];
        const float span = tau1 - tau0;
        const bool empty = !(e0 <= e1);
        const float dmax = fmaxf(fmaxf(fabsf(r.dx), fabsf(r.dy)), fabsf(r.dz));
        const float wt = dmax > 0.f ? widen / dmax : 0.f;
        T[i * 2 + 0] = (hit && !empty) ? (e0 - wt - tau0) / span : 1.f;
        T[i * 2 + 1] = (hit && !empty) ? (e1 + wt - tau0) / span : 0.f;
        valid[i] = hit ? 1 : 0;
    }
}

// ------------------------------------------------------------ fp32 forward
// out[r] = W3 relu(W2 relu(W1 x + b1) + b2) + b3, one thread per ray.
__global__ void __launch_bounds__(128) proposal_forward_kernel(const float* __restrict__ P,
                                                               const float* __restrict__ X, long long n,
                                                               float* __restrict__ out) {
    __shared__ float sW1[64 * 65], sW2[64 * 65];
    for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) {
        sW1[(i >> 6) * 65 + (i & 63)] = P[kPropW1 + i];
        sW2[(i >> 6) * 65 + (i & 63)] = P[kPropW2 + i];
    }
    __syncthreads();
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        float x[64], h[64];
        for (int k = 0; k < 64; ++k) x[k] = X[r * 64 + k];
        for (int o = 0; o < 64; ++o) {
            float a = P[kPropB1 + o];
            for (int k = 0; k < 64; ++k) a = fmaf(sW1[o * 65 + k], x[k], a);
            h[o] = fmaxf(a, 0.f);
        }
        for (int o = 0; o < 64; ++o) {
            float a = P[kPropB2 + o];
            for (int k = 0; k < 64; ++k) a = fmaf(sW2[o * 65 + k], h[k], a);
            x[o] = fmaxf(a, 0.f);
        }
        for (int o = 0; o < 2; ++o) {
            float a = P[kPropB3 + o];
            for (int k = 0; k < 64; ++k) a = fmaf(P[kPropW3 + o * 64 + k], x[k], a);
            out[r * 2 + o] = a;
        }
    }
}

// --------------------------------------------------------- fused training
// For a chunk of 64 rays per iteration (4 threads per ray, 256 threads):
//   forward  h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = W3 h2 + b3
//   loss     alpha * relu(e)^2 + relu(-e)^2 per end, with e the amount by
//            which the prediction clips the target interval (e_near =
//            y0 - t0, e_far = t1 - y1), so clipping costs alpha times more;
//            relu(y1 - y0 + kEmptyMargin)^2 for a ray with an empty target
//   backward dy, dh2 = (W3^T dy) * [h2 > 0], dh1 = (W2^T dh2) * [h1 > 0]
//   grads    dW1 += dh1 x^T, dW2 += dh2 h1^T, dW3 += dy h2^T, db = sums
// Each thread owns 16 entries of dW1 and of dW2 in registers across all its
// chunks; CTA results are added to `grads` with one atomic per entry.
constexpr int kTrainRays = 64;
// Target gap y0 - y1 (in units of the box span) for rays with nothing to march.
constexpr float kEmptyMargin = 0.05f;
constexpr int kLd = 65;

__global__ void __launch_bounds__(256) proposal_train_kernel(const float* __restrict__ P,
                                                             const float* __restrict__ X,
                                                             const float* __restrict__ T,
                                                             const uint8_t* __restrict__ valid, long long n,
                                                             float alpha, float inv_count, float* __restrict__ G,
                                                             float* __restrict__ loss) {
    extern __shared__ float sm[];
    float* sW1 = sm;                      // [64][65]
    float* sW2 = sW1 + 64 * kLd;          // [64][65]
    float* sW3 = sW2 + 64 * kLd;          // [2][64]
    float* sX = sW3 + 128;                // [64 rays][65]
    float* sH1 = sX + kTrainRays * kLd;
    float* sH2 = sH1 + kTrainRays * kLd;
    float* sD1 = sH2 + kTrainRays * kLd;  // dh1
    float* sD2 = sD1 + kTrainRays * kLd;  // dh2
    float* sDY = sD2 + kTrainRays * kLd;  // [64][2]
    float* sB = sDY + kTrainRays * 2;     // b1 [64], b2 [64], b3 [2]
    const int tid = threadIdx.x;
    for (int i = tid; i < 64 * 64; i += blockDim.x) {
        sW1[(i >> 6) * kLd + (i & 63)] = P[kPropW1 + i];
        sW2[(i >> 6) * kLd + (i & 63)] = P[kPropW2 + i];
    }
    for (int i = tid; i < 128; i += blockDim.x) sW3[i] = P[kPropW3 + i];
    for (int i = tid; i < 64; i += blockDim.x) {
        sB[i] = P[kPropB1 + i];
        sB[64 + i] = P[kPropB2 + i];
    }
    if (tid < 2) sB[128 + tid] = P[kPropB3 + tid];
    __syncthreads();

    // register-resident gradient accumulators
    const int go = tid >> 2, gi0 = (tid & 3) * 16;  // dW1/dW2 row go, columns gi0..gi0+15
    float gW1[16], gW2[16];
    for (int j = 0; j < 16; ++j) gW1[j] = gW2[j] = 0.f;
    float gB1 = 0.f, gB2 = 0.f, gW3 = 0.f, gB3 = 0.f;  // tid < 64: b1[tid], b2[tid]; tid < 128: W3; tid < 2: b3
    float lsum = 0.f;

    const int rr = tid >> 2, part = tid & 3;  // ray within the chunk, quarter of the outputs
    for (long long base = (long long)blockIdx.x * kTrainRays; base < n; base += (long long)gridDim.x * kTrainRays) {
        const long long r = base + rr;
        const bool ok = r < n && valid[r];
        // stage x
        for (int k = part; k < 64; k += 4) sX[rr * kLd + k] = ok ? X[r * 64 + k] : 0.f;
        __syncthreads();
        // h1 (this thread: outputs part*16 .. +15)
        for (int j = 0; j < 16; ++j) {
            const int o = part * 16 + j;
            float a = sB[o];
            for (int k = 0; k < 64; ++k) a = fmaf(sW1[o * kLd + k], sX[rr * kLd + k], a);
            sH1[rr * kLd + o] = fmaxf(a, 0.f);
        }
        __syncthreads();
        for (int j = 0; j < 16; ++j) {
            const int o = part * 16 + j;
            float a = sB[64 + o];
            for (int k = 0; k < 64; ++k) a = fmaf(sW2[o * kLd + k], sH1[rr * kLd + k], a);
            sH2[rr * kLd + o] = fmaxf(a, 0.f);
        }
        __syncthreads();
        if (part == 0) {
            float y[2];
            for (int o = 0; o < 2; ++o) {
                float a = sB[128 + o];
                for (int k = 0; k < 64; ++k) a = fmaf(sW3[o * 64 + k], sH2[rr * kLd + k], a);
                y[o] = a;
            }
            float dy0 = 0.f, dy1 = 0.f;
            if (ok && T[r * 2 + 0] > T[r * 2 + 1]) {
                // Empty ray: any proposal with y0 > y1 skips it whole and none
                // clips anything, so only a proposed window (y1 > y0 -
                // kEmptyMargin) costs, in samples of air marched.
                const float e = y[1] - y[0] + kEmptyMargin;
                if (e > 0.f) {
                    lsum += e * e;
                    dy0 = -2.f * e * inv_count;
                    dy1 = 2.f * e * inv_count;
                }
            } else if (ok) {
                const float en = y[0] - T[r * 2 + 0];  // > 0 clips the near end
                const float ef = T[r * 2 + 1] - y[1];  // > 0 clips the far end
                const float wn = en > 0.f ? alpha : 1.f, wf = ef > 0.f ? alpha : 1.f;
                lsum += wn * en * en + wf * ef * ef;
                dy0 = 2.f * wn * en * inv_count;
                dy1 = -2.f * wf * ef * inv_count;
            }
            sDY[rr * 2 + 0] = dy0;
            sDY[rr * 2 + 1] = dy1;
        }
        __syncthreads();
        // dh2 = W3^T dy masked by h2 > 0
        for (int j = 0; j < 16; ++j) {
            const int h = part * 16 + j;
            const float d = sW3[h] * sDY[rr * 2] + sW3[64 + h] * sDY[rr * 2 + 1];
            sD2[rr * kLd + h] = sH2[rr * kLd + h] > 0.f ? d : 0.f;
        }
        __syncthreads();
        // dh1 = W2^T dh2 masked by h1 > 0
        for (int j = 0; j < 16; ++j) {
            const int h = part * 16 + j;
            float a = 0.f;
            for (int o = 0; o < 64; ++o) a = fmaf(sW2[o * kLd + h], sD2[rr * kLd + o], a);
            sD1[rr * kLd + h] = sH1[rr * kLd + h] > 0.f ? a : 0.f;
        }
        __syncthreads();
        // weight gradients over the chunk's 64 rays
        for (int q = 0; q < kTrainRays; ++q) {
            const float d1 = sD1[q * kLd + go], d2 = sD2[q * kLd + go];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                gW1[j] = fmaf(d1, sX[q * kLd + gi0 + j], gW1[j]);
                gW2[j] = fmaf(d2, sH1[q * kLd + gi0 + j], gW2[j]);
            }
        }
        if (tid < 64) {
            for (int q = 0; q < kTrainRays; ++q) {
                gB1 += sD1[q * kLd + tid];
                gB2 += sD2[q * kLd + tid];
            }
        }
        if (tid < 128) {
            const int o = tid >> 6, h = tid & 63;
            for (int q = 0; q < kTrainRays; ++q) gW3 = fmaf(sDY[q * 2 + o], sH2[q * kLd + h], gW3);
        }
        if (tid < 2) {
            for (int q = 0; q < kTrainRays; ++q) gB3 += sDY[q * 2 + tid];
        }
        __syncthreads();
    }
    for (int j = 0; j < 16; ++j) {
        atomicAdd(G + kPropW1 + go * 64 + gi0 + j, gW1[j]);
        atomicAdd(G + kPropW2 + go * 64 + gi0 + j, gW2[j]);
    }
    if (tid < 64) {
        atomicAdd(G + kPropB1 + tid, gB1);
        atomicAdd(G + kPropB2 + tid, gB2);
    }
    if (tid < 128) atomicAdd(G + kPropW3 + tid, gW3);
    if (tid < 2) atomicAdd(G + kPropB3 + tid, gB3);
    // loss: warp sums then one atomic per warp
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0) atomicAdd(loss, lsum * inv_count);
}

constexpr size_t kTrainSmem = (size_t)(64 * kLd * 2 + 128 + kTrainRays * kLd * 5 + kTrainRays * 2 + 130) * 4;

// ------------------------------------------------------------------ Adam
__global__ void proposal_adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ m1,
                                     float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1,
                                     float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float g = G[i];
        const float a = b1 * m1[i] + (1.f - b1) * g;
        const float v = b2 * m2[i] + (1.f - b2) * g * g;
        m1[i] = a;
        m2[i] = v;
        P[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
    }
}

// ------------------------------------------------------------------ packing
__global__ void proposal_pack_kernel(const float* __restrict__ P, unsigned char* __restrict__ out) {
    __nv_bfloat16* w = reinterpret_cast<__nv_bfloat16*>(out);
    float* bias = reinterpret_cast<float*>(out + kPackB1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 64 * 64 + 64 * 64 + 8 * 64 + 136;
         i += gridDim.x * blockDim.x) {
        if (i < 4096) {
            w[i] = __float2bfloat16_rn(P[kPropW1 + i]);
        } else if (i < 8192) {
            w[i] = __float2bfloat16_rn(P[kPropW2 + i - 4096]);
        } else if (i < 8192 + 512) {
            const int j = i - 8192, row = j >> 6;
            w[i] = __float2bfloat16_rn(row < 2 ? P[kPropW3 + j] : 0.f);
        } else {
            const int j = i - 8192 - 512;  // 0..135
            bias[j] = j < 64 ? P[kPropB1 + j] : (j < 128 ? P[kPropB2 + j - 64] : (j < 130 ? P[kPropB3 + j - 128] : 0.f));
        }
    }
}

}  // namespace ndrr

// ==================================================================== C ABI
namespace {
thread_local char g_prop_msg[256];
int32_t prop_fail(int32_t code, const char* msg) {
    snprintf(g_prop_msg, sizeof(g_prop_msg), "%s", msg);
    return code;
}
int32_t prop_cuda(cudaError_t e) {
    if (e == cudaSuccess) return NDRR_OK;
    snprintf(g_prop_msg, sizeof(g_prop_msg), "CUDA error: %s", cudaGetErrorString(e));
    return NDRR_ERR_CUDA;
}
int prop_grid(long long n, int block) { return (int)std::max(1LL, std::min((n + block - 1) / block, 152LL * 16)); }
}  // namespace

extern "C" {

NDRR_API const char* ndrr_proposal_last_error(void) { return g_prop_msg; }

NDRR_API int32_t ndrr_proposal_dataset(const ndrr_raymarch_args* a, const float* extent, float widen_voxels,
                                       float* features, float* targets, uint8_t* valid, void* stream) {
    if (!a || !extent || !features || !targets || !valid) return prop_fail(NDRR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (a->B <= 0 || a->N <= 0) return NDRR_OK;
    if (!a->M || !a->src || !a->tgt) return prop_fail(NDRR_ERR_INVALID_ARGUMENT, "M, src, tgt must be non-NULL");
    const long long total = (long long)a->B * a->N;
    ndrr::proposal_dataset_kernel<<<prop_grid(total, 256), 256, 0, (cudaStream_t)stream>>>(
        a->M, a->src, a->tgt, a->src_per_ray, a->B, a->N, a->D, a->H, a->W, extent, widen_voxels, features, targets,
        valid);
    return prop_cuda(cudaGetLastError());
}

NDRR_API int32_t ndrr_proposal_train_step(const float* params, const float* features, const float* targets,
                                          const uint8_t* valid, int64_t n, float alpha, float inv_count,
                                          float* grads, float* loss, void* stream) {
    if (!params || !features || !targets || !valid || !grads || !loss)
        return prop_fail(NDRR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n <= 0) return NDRR_OK;
    const cudaError_t ea = cudaFuncSetAttribute(ndrr::proposal_train_kernel,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ndrr::kTrainSmem);
    if (ea != cudaSuccess) return prop_cuda(ea);
    const int grid = (int)std::max(1LL, std::min(((long long)n + ndrr::kTrainRays - 1) / ndrr::kTrainRays, 152LL * 2));
    ndrr::proposal_train_kernel<<<grid, 256, ndrr::kTrainSmem, (cudaStream_t)stream>>>(
        params, features, targets, valid, (long long)n, alpha, inv_count, grads, loss);
    return prop_cuda(cudaGetLastError());
}

NDRR_API int32_t ndrr_proposal_forward(const float* params, const float* features, int64_t n, float* out,
                                       void* stream) {
    if (!params || !features || !out) return prop_fail(NDRR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n <= 0) return NDRR_OK;
    ndrr::proposal_forward_kernel<<<prop_grid(n, 128), 128, 0, (cudaStream_t)stream>>>(params, features, (long long)n,
                                                                                       out);
    return prop_cuda(cudaGetLastError());
}

NDRR_API int32_t ndrr_proposal_adam(float* params, const float* grads, float* m1, float* m2, int32_t step, float lr,
                                    float beta1, float beta2, float eps, void* stream) {
    if (!params || !grads || !m1 || !m2 || step < 1) return prop_fail(NDRR_ERR_INVALID_ARGUMENT, "bad argument");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    ndrr::proposal_adam_kernel<<<prop_grid(ndrr::kPropParams, 256), 256, 0, (cudaStream_t)stream>>>(
        params, grads, m1, m2, ndrr::kPropParams, lr, beta1, beta2, eps, c1, c2);
    return prop_cuda(cudaGetLastError());
}

NDRR_API int32_t ndrr_proposal_pack(const float* params, void* packed, void* stream) {
    if (!params || !packed) return prop_fail(NDRR_ERR_INVALID_ARGUMENT, "NULL argument");
    ndrr::proposal_pack_kernel<<<8, 256, 0, (cudaStream_t)stream>>>(params, (unsigned char*)packed);
    return prop_cuda(cudaGetLastError());
}

}  // extern "C"
