// Empty-space sample windows computed ahead of the march (ndrr_skip_windows).
//
// Running the network inside the render kernels would cost the whole march
// occupancy (19.7 KB of shared memory for the weights per CTA, and the
// fragment registers); measured that way the learned forward took 6.0 ms
// against 0.7 + 1.8 ms here. So the network and the occupancy check run once
// per ray in their own persistent kernel and leave each ray's sample window
// [lo, hi) in a [B, N, 2] int32 buffer (8 bytes per ray), which the plain
// march kernels read in their ray set-up; the forward and the adjoint of one
// step share it. The occupancy skip computes the same windows (apply_skip)
// either here or inside the march.
#include "ndrr_march.cuh"

namespace ndrr {

constexpr int kWinRays = 128;  // rays per work item: four warps, one network tile each

template <int MODE>
__global__ void __launch_bounds__(kWinRays) skip_windows_kernel(const MarchParams p, int* __restrict__ win) {
    extern __shared__ __align__(16) unsigned char wsm[];
    if (MODE == NDRR_SKIP_PROPOSAL) proposal_stage_weights(p.proposal, wsm);
    const long long total = (long long)p.B * p.N;
    const long long items = (total + kWinRays - 1) / kWinRays;
    for (long long item = blockIdx.x; item < items; item += gridDim.x) {
        const long long g = item * kWinRays + threadIdx.x;
        const bool valid = g < total;
        const int b = valid ? (int)(g / p.N) : 0;
        const int n = valid ? (int)(g - (long long)b * p.N) : -1;
        float m[12];
#pragma unroll
        for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
        ThreadRay tr;
        init_thread_ray(p, m, b, n, tr);
        const int box_len = max(tr.ray.hi - tr.ray.lo, 0);
        const bool has = n >= 0 && box_len > 0;
        float pn = 0.f, pf = 1.f;
        // all threads take part (the proposal synchronises the CTA)
        if (MODE == NDRR_SKIP_PROPOSAL)
            proposal_window_cta(wsm, tr.ray, p.D, p.H, p.W, has, threadIdx.x, 0, kWinRays, pn, pf);
        const bool fell = apply_skip(p, tr, pn, pf);
        if (p.stats) skip_stats_add(p, p.stats, 0, has, fell, box_len, max(tr.ray.hi - tr.ray.lo, 0));
        if (valid) {
            int2 w;
            w.x = tr.ray.lo;
            w.y = max(tr.ray.hi, tr.ray.lo);
            reinterpret_cast<int2*>(win)[g] = w;
        }
    }
}

template <int MODE>
static cudaError_t launch_windows_mode(const MarchParams& p, int* win, cudaStream_t st) {
    const size_t smem = MODE == NDRR_SKIP_PROPOSAL ? proposal_smem_bytes(kWinRays) : 0;
    const long long total = (long long)p.B * p.N;
    const unsigned items = (unsigned)((total + kWinRays - 1) / kWinRays);
    auto kern = skip_windows_kernel<MODE>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWinRays, smem);
    if (e != cudaSuccess) return e;
    const unsigned cap = (unsigned)std::max(1, sms * std::max(per_sm, 1));
    kern<<<std::min(items, cap), kWinRays, smem, st>>>(p, win);
    return cudaGetLastError();
}

cudaError_t launch_skip_windows(const ndrr_raymarch_args& a, int32_t* windows, cudaStream_t st) {
    LaunchShape ls;  // tile fields unused: the window kernel indexes rays linearly
    MarchParams p = make_params(a, ls);
    p.win = nullptr;
    if (a.skip_mode == NDRR_SKIP_PROPOSAL) return launch_windows_mode<NDRR_SKIP_PROPOSAL>(p, windows, st);
    return launch_windows_mode<NDRR_SKIP_OCCUPANCY>(p, windows, st);
}

}  // namespace ndrr
