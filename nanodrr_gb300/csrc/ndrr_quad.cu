// Volume preparation and the quad layout: the HU -> attenuation conversion,
// the quad build (one pass over the padded extent) and the fold of the
// quad-layout volume gradient back into the volume's layout. The layout is
// defined in ndrr_device.cuh (QuadOf, make_quadgeom).
#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT>
__device__ __forceinline__ VT ld_raw(const VT* p, long long idx) {
    return p[idx];
}

// 32-bit float volume -> float4 quads.
__global__ void quad_build_f32_kernel(const float* __restrict__ v, int D, int H, int W, float4* __restrict__ q) {
    const int QX = W + 3, QY = H + 3;
    const long long n = (long long)(D + 4) * QY * QX;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int qx = (int)(i % QX), qy = (int)((i / QX) % QY), qz = (int)(i / ((long long)QX * QY));
        const int x0 = qx - 2, y0 = qy - 2, z = qz - 2;
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        if ((unsigned)z < (unsigned)D) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int x = x0 + (k & 1), y = y0 + (k >> 1);
                if ((unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H) c[k] = v[((size_t)z * H + y) * W + x];
            }
        }
        q[i] = make_float4(c[0], c[1], c[2], c[3]);
    }
}

// 16-bit volume -> four raw 16-bit values per quad (bit-exact copies).
__global__ void quad_build_b16_kernel(const uint16_t* __restrict__ v, int D, int H, int W, uint2* __restrict__ q) {
    const int QX = W + 3, QY = H + 3;
    const long long n = (long long)(D + 4) * QY * QX;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int qx = (int)(i % QX), qy = (int)((i / QX) % QY), qz = (int)(i / ((long long)QX * QY));
        const int x0 = qx - 2, y0 = qy - 2, z = qz - 2;
        uint32_t c[4] = {0u, 0u, 0u, 0u};
        if ((unsigned)z < (unsigned)D) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int x = x0 + (k & 1), y = y0 + (k >> 1);
                if ((unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H) c[k] = v[((size_t)z * H + y) * W + x];
            }
        }
        q[i] = make_uint2(c[0] | (c[1] << 16), c[2] | (c[3] << 16));
    }
}

// 16-bit volume + label map -> labelled quads: the four raw 16-bit corner
// values as in quad_build_b16_kernel, and the four corners' classes (class
// in [0, C) as uint8, 255 for a label outside it; 0 for a corner outside the
// volume, the class the nearest-label rule gives a position there).
__global__ void quad_build_labeled_kernel(const uint16_t* __restrict__ v, const void* __restrict__ lab,
                                          int lab_dtype, int C, int D, int H, int W, uint4* __restrict__ q) {
    const int QX = W + 3, QY = H + 3;
    const long long n = (long long)(D + 4) * QY * QX;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int qx = (int)(i % QX), qy = (int)((i / QX) % QY), qz = (int)(i / ((long long)QX * QY));
        const int x0 = qx - 2, y0 = qy - 2, z = qz - 2;
        uint32_t c[4] = {0u, 0u, 0u, 0u};
        uint32_t labels = 0u;
        if ((unsigned)z < (unsigned)D) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int x = x0 + (k & 1), y = y0 + (k >> 1);
                if ((unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H) {
                    const int idx = (z * H + y) * W + x;
                    c[k] = v[idx];
                    const int cls = ld_label(lab, lab_dtype, idx);
                    labels |= (uint32_t)((unsigned)cls < (unsigned)C ? cls : 255) << (8 * k);
                }
            }
        }
        q[i] = make_uint4(c[0] | (c[1] << 16), c[2] | (c[3] << 16), labels, 0u);
    }
}

// gvol[z][y][x] += the four quad entries in which voxel (x, y) of plane z is
// a corner: (x, y) as (x0, y0), (x0 + 1, y0), (x0, y0 + 1), (x0 + 1, y0 + 1).
// One CTA per kFoldRows consecutive lines (z, y) of the volume, four
// consecutive x per thread: the five quad entries of a quad row are 16-byte
// loads, and walking down the lines each quad row is loaded once and serves
// as the upper row of one line and the lower row of the next.
constexpr int kFoldRows = 8;

template <bool OVERWRITE>
__global__ void __launch_bounds__(128) quad_fold_kernel(const float4* __restrict__ gq, int D, int H, int W,
                                                        float* __restrict__ gvol) {
    const int QX = W + 3, QY = H + 3;
    const int nyb = (H + kFoldRows - 1) / kFoldRows;
    const int z = (int)(blockIdx.x / (unsigned)nyb), y0 = (int)(blockIdx.x % (unsigned)nyb) * kFoldRows;
    const int y1 = min(H, y0 + kFoldRows);
    const bool vec = (W & 3) == 0;
    for (int x0 = threadIdx.x * 4; x0 < W; x0 += blockDim.x * 4) {
        // entries x0 + 1 .. x0 + 5 (all inside the padded row of W + 3)
        int e[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) e[k] = min(x0 + 1 + k, QX - 1);
        const float4* row = gq + ((size_t)(z + 2) * QY + (y0 + 1)) * QX;  // entries with y0 = y - 1
        float4 c[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) c[k] = __ldg(row + e[k]);
        for (int y = y0; y < y1; ++y) {
            row += QX;  // entries with y0 = y
            float4 a[5];
#pragma unroll
            for (int k = 0; k < 5; ++k) a[k] = __ldg(row + e[k]);
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = (a[j + 1].x + a[j].y) + (c[j + 1].z + c[j].w);
            float* out = gvol + ((size_t)z * H + y) * W;
            if (vec) {
                float4 o = OVERWRITE ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<float4*>(out + x0);
                o.x += v[0];
                o.y += v[1];
                o.z += v[2];
                o.w += v[3];
                *reinterpret_cast<float4*>(out + x0) = o;
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (x0 + j < W) out[x0 + j] = OVERWRITE ? v[j] : out[x0 + j] + v[j];
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) c[k] = a[k];
        }
    }
}

// HU -> linear attenuation (1/mm), the reference's piecewise-linear map
// (nanodrr src/nanodrr/data/preprocess.py:44-50): clamp HU at -1000; at or
// below 0 HU the air-water line (h / 1000 + 1) * mu_water, above it the
// water-bone line mu_water + (h / hu_bone) * dmu with dmu = mu_bone -
// mu_water; clamp at 0 (NaN passes through both clamps, as torch.clamp lets
// it). One element per thread and grid-stride, in fp32; the
// 16-bit types convert on load and round to nearest-even on store.
template <typename T>
__device__ __forceinline__ float hu_load(const T* p, long long i);
template <>
__device__ __forceinline__ float hu_load<float>(const float* p, long long i) { return __ldg(p + i); }
template <>
__device__ __forceinline__ float hu_load<__half>(const __half* p, long long i) { return __half2float(__ldg(p + i)); }
template <>
__device__ __forceinline__ float hu_load<__nv_bfloat16>(const __nv_bfloat16* p, long long i) {
    return __bfloat162float(__ldg(p + i));
}

template <typename T>
__global__ void __launch_bounds__(256) hu_to_mu_kernel(const T* __restrict__ hu, long long n, float mu_water,
                                                       float dmu, float hu_bone, T* __restrict__ mu) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float x = hu_load(hu, i);
        const float h = x < -1000.0f ? -1000.0f : x;  // NaN stays NaN, as in torch.clamp
        const float below = __fmul_rn(__fadd_rn(__fdiv_rn(h, 1000.0f), 1.0f), mu_water);
        const float above = __fadd_rn(mu_water, __fmul_rn(__fdiv_rn(h, hu_bone), dmu));
        const float m = h > 0.0f ? above : below;
        st_out(mu, (size_t)i, m > 0.0f ? m : (m == m ? 0.0f : m));
    }
}

static int grid_for(long long n) { return (int)std::max(1LL, std::min((n + 255) / 256, 152LL * 32)); }

cudaError_t launch_quad_build(const void* vol, int dtype, int D, int H, int W, void* quad, cudaStream_t st) {
    const long long n = (long long)(D + 4) * (H + 3) * (W + 3);
    if (dtype == NDRR_F32)
        quad_build_f32_kernel<<<grid_for(n), 256, 0, st>>>((const float*)vol, D, H, W, (float4*)quad);
    else if (dtype == NDRR_F16 || dtype == NDRR_BF16)
        quad_build_b16_kernel<<<grid_for(n), 256, 0, st>>>((const uint16_t*)vol, D, H, W, (uint2*)quad);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_quad_build_labeled(const void* vol, int dtype, const void* lab, int lab_dtype, int C, int D, int H,
                                      int W, void* quad, cudaStream_t st) {
    if (dtype != NDRR_F16 && dtype != NDRR_BF16) return cudaErrorInvalidValue;
    const long long n = (long long)(D + 4) * (H + 3) * (W + 3);
    quad_build_labeled_kernel<<<grid_for(n), 256, 0, st>>>((const uint16_t*)vol, lab, lab_dtype, C, D, H, W,
                                                           (uint4*)quad);
    return cudaGetLastError();
}

cudaError_t launch_hu_to_mu(const void* hu, int dtype, long long n, float mu_water, float dmu, float hu_bone,
                            void* mu, cudaStream_t st) {
    switch (dtype) {
        case NDRR_F32:
            hu_to_mu_kernel<<<grid_for(n), 256, 0, st>>>((const float*)hu, n, mu_water, dmu, hu_bone, (float*)mu);
            break;
        case NDRR_F16:
            hu_to_mu_kernel<<<grid_for(n), 256, 0, st>>>((const __half*)hu, n, mu_water, dmu, hu_bone, (__half*)mu);
            break;
        case NDRR_BF16:
            hu_to_mu_kernel<<<grid_for(n), 256, 0, st>>>((const __nv_bfloat16*)hu, n, mu_water, dmu, hu_bone,
                                                         (__nv_bfloat16*)mu);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_quad_fold(const float* gquad, int D, int H, int W, float* gvol, bool overwrite,
                             cudaStream_t st) {
    const unsigned grid = (unsigned)((long long)D * ((H + kFoldRows - 1) / kFoldRows));
    if (overwrite)
        quad_fold_kernel<true><<<grid, 128, 0, st>>>((const float4*)gquad, D, H, W, gvol);
    else
        quad_fold_kernel<false><<<grid, 128, 0, st>>>((const float4*)gquad, D, H, W, gvol);
    return cudaGetLastError();
}

}  // namespace ndrr
