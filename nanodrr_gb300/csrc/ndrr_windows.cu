// Empty-space sample windows computed ahead of the march (ndrr_skip_windows).
//
// Running the network inside the render kernels would cost the whole march
// occupancy (19.7 KB of shared memory for the weights per CTA, and the
// fragment registers); measured that way the learned forward took 6.0 ms
// against 0.7 + 1.8 ms here. So the network and the occupancy check run once
// per ray ahead of the march and leave each ray's sample window [lo, hi) in a
// [B, N, 2] int32 buffer (8 bytes per ray), which the plain march kernels
// read in their ray set-up; the forward and the adjoint of one step share it.
//
// The learned proposal takes two launches over the same buffer: the network
// kernel (shared-memory weights, CTA-wide tensor-core tiles) writes each
// ray's proposed [pn, pf] as float bits, and the check kernel (no shared
// memory, full occupancy, no CTA barrier) walks the distance field and
// overwrites them with the window. In one kernel the walks ran at the
// network's occupancy (5 CTAs per SM) and every tile waited for its longest
// walk: on a phantom with much air (long empty walks) that cost 3.5 ms for
// 2.1 M rays against 0.3 ms for the occupancy windows alone. The occupancy
// skip computes the same windows (apply_skip) in the check kernel alone, or
// inside the march.
#include "ndrr_march.cuh"

namespace ndrr {

constexpr int kWinRays = 128;  // rays per work item: four warps, one network tile each

__device__ __forceinline__ void window_ray(const MarchParams& p, long long g, ThreadRay& tr, int& b, int& n) {
    const long long total = (long long)p.B * p.N;
    const bool valid = g < total;
    b = valid ? (int)(g / p.N) : 0;
    n = valid ? (int)(g - (long long)b * p.N) : -1;
    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
    init_thread_ray(p, m, b, n, tr);
}

// Network pass: proposed [pn, pf] (in t, as float bits) for every ray.
__global__ void __launch_bounds__(kWinRays) proposal_windows_kernel(const MarchParams p, int* __restrict__ win) {
    extern __shared__ __align__(16) unsigned char wsm[];
    proposal_stage_weights(p.proposal, wsm);
    const long long total = (long long)p.B * p.N;
    const long long items = (total + kWinRays - 1) / kWinRays;
    for (long long item = blockIdx.x; item < items; item += gridDim.x) {
        const long long g = item * kWinRays + threadIdx.x;
        ThreadRay tr;
        int b, n;
        window_ray(p, g, tr, b, n);
        const bool has = n >= 0 && tr.ray.hi > tr.ray.lo;
        float pn = 0.f, pf = 1.f;
        // all threads take part (the network synchronises the CTA)
        proposal_window_cta(wsm, tr.ray, p.D, p.H, p.W, has, threadIdx.x, 0, kWinRays, pn, pf);
        if (g < total) reinterpret_cast<int2*>(win)[g] = make_int2(__float_as_int(pn), __float_as_int(pf));
    }
}

// Check pass (MODE NDRR_SKIP_PROPOSAL: reads the proposals in `win`) or the
// whole occupancy skip (NDRR_SKIP_OCCUPANCY); writes the windows into `win`.
template <int MODE>
__global__ void __launch_bounds__(kWinRays) skip_windows_kernel(const MarchParams p, int* __restrict__ win) {
    const long long total = (long long)p.B * p.N;
    for (long long g = (long long)blockIdx.x * kWinRays + threadIdx.x; g - threadIdx.x < total;
         g += (long long)gridDim.x * kWinRays) {
        const bool valid = g < total;
        ThreadRay tr;
        int b, n;
        window_ray(p, g, tr, b, n);
        const int box_len = max(tr.ray.hi - tr.ray.lo, 0);
        const bool has = n >= 0 && box_len > 0;
        float pn = 0.f, pf = 1.f;
        if (MODE == NDRR_SKIP_PROPOSAL && valid) {
            const int2 pr = reinterpret_cast<const int2*>(win)[g];
            pn = __int_as_float(pr.x);
            pf = __int_as_float(pr.y);
        }
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

// Persistent grid: CTAs resident at once, at most one per work item.
template <typename Kern>
static cudaError_t persistent_grid(Kern kern, size_t smem, unsigned items, unsigned& grid) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWinRays, smem);
    if (e != cudaSuccess) return e;
    grid = std::min(items, (unsigned)std::max(1, sms * std::max(per_sm, 1)));
    return cudaSuccess;
}

cudaError_t launch_skip_windows(const ndrr_raymarch_args& a, int32_t* windows, cudaStream_t st) {
    LaunchShape ls;  // tile fields unused: the window kernels index rays linearly
    MarchParams p = make_params(a, ls);
    p.win = nullptr;
    const long long total = (long long)p.B * p.N;
    const unsigned items = (unsigned)((total + kWinRays - 1) / kWinRays);
    unsigned grid = 0;
    cudaError_t e;
    if (a.skip_mode == NDRR_SKIP_PROPOSAL) {
        const size_t smem = proposal_smem_bytes(kWinRays);
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(proposal_windows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        if ((e = persistent_grid(proposal_windows_kernel, smem, items, grid)) != cudaSuccess) return e;
        proposal_windows_kernel<<<grid, kWinRays, smem, st>>>(p, windows);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = persistent_grid(skip_windows_kernel<NDRR_SKIP_PROPOSAL>, 0, items, grid)) != cudaSuccess) return e;
        skip_windows_kernel<NDRR_SKIP_PROPOSAL><<<grid, kWinRays, 0, st>>>(p, windows);
        return cudaGetLastError();
    }
    if ((e = persistent_grid(skip_windows_kernel<NDRR_SKIP_OCCUPANCY>, 0, items, grid)) != cudaSuccess) return e;
    skip_windows_kernel<NDRR_SKIP_OCCUPANCY><<<grid, kWinRays, 0, st>>>(p, windows);
    return cudaGetLastError();
}

}  // namespace ndrr
