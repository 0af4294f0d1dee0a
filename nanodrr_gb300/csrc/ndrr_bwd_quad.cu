// Adjoint instantiations for the quad volume layout: quad gathers, and the
// volume gradient scattered into the quad-layout gradient.
#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT, bool MULTI, bool GCAM>
static cudaError_t bwd_quad_skip(const MarchParams& p, int skip, unsigned grid, unsigned block, size_t smem,
                                 cudaStream_t st) {
    if (skip == NDRR_SKIP_OCCUPANCY)
        return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, GCAM, 1, true>, grid, block, smem, st, p);
    return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, GCAM, 0, true>, grid, block, smem, st, p);
}

template <typename VT, bool MULTI>
static cudaError_t bwd_quad_flags(const MarchParams& p, bool gvol, bool gcam, int skip, unsigned grid,
                                  unsigned block, size_t smem, cudaStream_t st) {
    if (gvol && gcam) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, true, 0, true>, grid, block, smem, st, p);
    if (gvol) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, false, 0, true>, grid, block, smem, st, p);
    if (gcam) return bwd_quad_skip<VT, MULTI, true>(p, skip, grid, block, smem, st);
    return bwd_quad_skip<VT, MULTI, false>(p, skip, grid, block, smem, st);
}

template <typename VT>
static cudaError_t bwd_quad_multi(const MarchParams& p, bool multi, bool gvol, bool gcam, int skip, unsigned grid,
                                  unsigned block, size_t smem, cudaStream_t st) {
    return multi ? bwd_quad_flags<VT, true>(p, gvol, gcam, skip, grid, block, smem, st)
                 : bwd_quad_flags<VT, false>(p, gvol, gcam, skip, grid, block, smem, st);
}

cudaError_t launch_bwd_quad(const MarchParams& p, int vol_dtype, bool multi, bool gvol, bool gcam, int skip,
                            unsigned grid, unsigned block, size_t smem, cudaStream_t st) {
    switch (vol_dtype) {
        case NDRR_F32: return bwd_quad_multi<float>(p, multi, gvol, gcam, skip, grid, block, smem, st);
        case NDRR_F16: return bwd_quad_multi<__half>(p, multi, gvol, gcam, skip, grid, block, smem, st);
        case NDRR_BF16: return bwd_quad_multi<__nv_bfloat16>(p, multi, gvol, gcam, skip, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ndrr
