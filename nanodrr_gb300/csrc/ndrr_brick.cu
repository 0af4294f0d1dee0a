// Launcher of the adjoint with the per-slab shared-memory volume-gradient
// brick (kernel in ndrr_march.cuh).
#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT, bool MULTI>
static cudaError_t brick_dispatch(const MarchParams& p, bool gcam, unsigned grid, unsigned block, size_t smem,
                                  cudaStream_t st, int cap, int L0) {
    auto kern = gcam ? raymarch_bwd_brick_kernel<VT, MULTI, true> : raymarch_bwd_brick_kernel<VT, MULTI, false>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, block, smem, st>>>(p, cap, L0);
    return cudaGetLastError();
}

cudaError_t launch_brick(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p, unsigned grid,
                         unsigned block, cudaStream_t st) {
    const size_t smem = brick_smem_bytes(a, ls);
    const bool multi = a.n_classes > 1, gcam = a.need_gcam != 0;
    switch (a.vol_dtype) {
        case NDRR_F32:
            return multi ? brick_dispatch<float, true>(p, gcam, grid, block, smem, st, ls.cap, ls.L0)
                         : brick_dispatch<float, false>(p, gcam, grid, block, smem, st, ls.cap, ls.L0);
        case NDRR_F16:
            return multi ? brick_dispatch<__half, true>(p, gcam, grid, block, smem, st, ls.cap, ls.L0)
                         : brick_dispatch<__half, false>(p, gcam, grid, block, smem, st, ls.cap, ls.L0);
        case NDRR_BF16:
            return multi ? brick_dispatch<__nv_bfloat16, true>(p, gcam, grid, block, smem, st, ls.cap, ls.L0)
                         : brick_dispatch<__nv_bfloat16, false>(p, gcam, grid, block, smem, st, ls.cap, ls.L0);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ndrr
