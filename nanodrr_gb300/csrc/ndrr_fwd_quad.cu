// Forward instantiations for the quad volume layout (output in the volume's
// dtype, every skip mode).
#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT, bool MULTI>
static cudaError_t fwd_quad_skip(const MarchParams& p, int skip, unsigned grid, unsigned block, size_t smem,
                                 cudaStream_t st) {
    if (skip == NDRR_SKIP_OCCUPANCY)
        return launch_kernel(raymarch_fwd_kernel<VT, VT, MULTI, 1, true>, grid, block, smem, st, p);
    return launch_kernel(raymarch_fwd_kernel<VT, VT, MULTI, 0, true>, grid, block, smem, st, p);
}

template <typename VT>
static cudaError_t fwd_quad_multi(const MarchParams& p, bool multi, int skip, unsigned grid, unsigned block,
                                  size_t smem, cudaStream_t st) {
    return multi ? fwd_quad_skip<VT, true>(p, skip, grid, block, smem, st)
                 : fwd_quad_skip<VT, false>(p, skip, grid, block, smem, st);
}

cudaError_t launch_fwd_quad(const MarchParams& p, int vol_dtype, bool multi, int skip, unsigned grid,
                            unsigned block, size_t smem, cudaStream_t st) {
    switch (vol_dtype) {
        case NDRR_F32: return fwd_quad_multi<float>(p, multi, skip, grid, block, smem, st);
        case NDRR_F16: return fwd_quad_multi<__half>(p, multi, skip, grid, block, smem, st);
        case NDRR_BF16: return fwd_quad_multi<__nv_bfloat16>(p, multi, skip, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ndrr
