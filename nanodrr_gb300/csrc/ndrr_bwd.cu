// Adjoint launcher: the direct-atomics adjoint kernels (with the skip modes
// for pose-only adjoints), the brick variant for volume gradients
// (ndrr_brick.cu) and the fixed-order per-pose reduction of the partials.
#include "ndrr_march.cuh"

namespace ndrr {

// Per-pose sum of the per-tile partials in a fixed order. One CTA per pose.
__global__ void __launch_bounds__(256) pose_partials_reduce_kernel(const float* __restrict__ partials, int tiles,
                                                                   float* __restrict__ gM,
                                                                   float* __restrict__ gsrc_shared) {
    __shared__ float red[8][16];
    const int b = blockIdx.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nterms = gsrc_shared ? 15 : 12;
    for (int j = 0; j < nterms; ++j) {
        float v = 0.f;
        for (int t = tid; t < tiles; t += blockDim.x) v += partials[((size_t)b * tiles + t) * kPartialStride + j];
        v = warp_sum(v);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (tid < nterms) {
        float sum = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += red[w][tid];
        if (tid < 12)
            gM[(size_t)b * 12 + tid] = sum;
        else
            gsrc_shared[(size_t)b * 3 + (tid - 12)] = sum;
    }
}

template <typename VT, bool MULTI, bool GCAM>
static cudaError_t bwd_dispatch_skip(const MarchParams& p, int skip, unsigned grid, unsigned block, size_t smem,
                                     cudaStream_t st) {
    if (skip == NDRR_SKIP_OCCUPANCY)
        return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, GCAM, 1, kLayoutVolume>, grid, block, smem, st, p);
    return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, GCAM, 0, kLayoutVolume>, grid, block, smem, st, p);
}

template <typename VT, bool MULTI>
static cudaError_t bwd_dispatch_flags(const MarchParams& p, bool gvol, bool gcam, int skip, unsigned grid,
                                      unsigned block, size_t smem, cudaStream_t st) {
    // With a volume gradient every sample matters: skipping never applies.
    if (gvol && gcam) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, true, 0, kLayoutVolume>, grid, block, smem, st, p);
    if (gvol) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, false, 0, kLayoutVolume>, grid, block, smem, st, p);
    if (gcam) return bwd_dispatch_skip<VT, MULTI, true>(p, skip, grid, block, smem, st);
    return bwd_dispatch_skip<VT, MULTI, false>(p, skip, grid, block, smem, st);
}

template <typename VT>
static cudaError_t bwd_dispatch(const MarchParams& p, bool multi, bool gvol, bool gcam, int skip, unsigned grid,
                                unsigned block, size_t smem, cudaStream_t st) {
    if (multi) return bwd_dispatch_flags<VT, true>(p, gvol, gcam, skip, grid, block, smem, st);
    return bwd_dispatch_flags<VT, false>(p, gvol, gcam, skip, grid, block, smem, st);
}

cudaError_t launch_bwd(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st) {
    MarchParams p = make_params(a, ls);
    const bool multi = a.n_classes > 1, gvol = a.need_gvol != 0, gcam = a.need_gcam != 0;
    const int skip = gvol ? NDRR_SKIP_NONE : a.skip_mode;
    unsigned grid = (unsigned)((size_t)a.B * p.tm.tiles);
    const unsigned block = (unsigned)(ls.tw * ls.th * ls.K);
    cudaError_t e;
    if (a.vol_quad != nullptr) {
        // quad-layout gathers; with a volume gradient the taps go to the
        // quad-layout gradient, zeroed here and folded into gvol below
        if (gvol) {
            e = cudaMemsetAsync(a.gvol_quad, 0, (size_t)(a.D + 4) * (a.H + 3) * (a.W + 3) * 16, st);
            if (e != cudaSuccess) return e;
        }
        if (gvol && ls.split) {
            // split adjoint: the pose pass (gathers; the call's skip or
            // sample windows drop only samples without pose terms), then
            // the positions-only scatter pass in slab order, then the fold.
            // The kernel events, when set, bracket both march passes.
            KernelEvents& ev = kernel_events();
            const KernelEvents outer = ev;
            ev = KernelEvents{};
            MarchParams pp = p;
            pp.partials = slab_partials(a, ls);
            if (outer.start != nullptr) cudaEventRecord(outer.start, st);
            e = launch_bwd_quad(pp, a.vol_dtype, false, false, false, a.skip_mode, a.quad_labels != 0, grid, block,
                                bwd_smem_bytes(a, ls), st);
            if (e == cudaSuccess) {
                pose_partials_reduce_kernel<<<a.B, 256, 0, st>>>(pp.partials, p.tm.tiles, a.gM, nullptr);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = launch_scatter_slab(a, ls, p, st);
            if (e == cudaSuccess && outer.stop != nullptr) e = cudaEventRecord(outer.stop, st);
            ev = outer;
            if (e == cudaSuccess) e = launch_quad_fold(a.gvol_quad, a.D, a.H, a.W, a.gvol, a.gvol_overwrite != 0, st);
            return e;
        }
        if (gvol && ls.slab) {
            // slab-ordered adjoint: writes gM itself (ndrr_slab.cu)
            e = launch_bwd_slab(a, ls, p, st);
            if (e == cudaSuccess) e = launch_quad_fold(a.gvol_quad, a.D, a.H, a.W, a.gvol, a.gvol_overwrite != 0, st);
            return e;
        }
        e = launch_bwd_quad(p, a.vol_dtype, multi, gvol, gcam, skip, a.quad_labels != 0, grid, block,
                            bwd_smem_bytes(a, ls), st);
        if (e == cudaSuccess && gvol) e = launch_quad_fold(a.gvol_quad, a.D, a.H, a.W, a.gvol, a.gvol_overwrite != 0, st);
    } else if (gvol && ls.brick) {
        e = launch_brick(a, ls, p, grid, block, st);
    } else {
        const size_t smem = bwd_smem_bytes(a, ls);
        switch (a.vol_dtype) {
            case NDRR_F32: e = bwd_dispatch<float>(p, multi, gvol, gcam, skip, grid, block, smem, st); break;
            case NDRR_F16: e = bwd_dispatch<__half>(p, multi, gvol, gcam, skip, grid, block, smem, st); break;
            case NDRR_BF16:
                e = bwd_dispatch<__nv_bfloat16>(p, multi, gvol, gcam, skip, grid, block, smem, st);
                break;
            default: return cudaErrorInvalidValue;
        }
    }
    if (e != cudaSuccess) return e;
    float* gsrc_shared = (a.need_gcam && !a.src_per_ray) ? a.gsrc : nullptr;
    pose_partials_reduce_kernel<<<a.B, 256, 0, st>>>(p.partials, p.tm.tiles, a.gM, gsrc_shared);
    return cudaGetLastError();
}

}  // namespace ndrr
