// Adjoint instantiations for the quad volume layouts: quad gathers, and the
// volume gradient scattered into the quad-layout gradient. The labelled quad
// layout (16-bit volumes with label channels) routes each sample by the class
// its two loads carry.
#include <type_traits>

#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT, bool MULTI, bool GCAM, int LAYOUT>
static cudaError_t bwd_quad_skip(const MarchParams& p, int skip, unsigned grid, unsigned block, size_t smem,
                                 cudaStream_t st) {
    if (skip == NDRR_SKIP_OCCUPANCY)
        return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, GCAM, 1, LAYOUT>, grid, block, smem, st, p);
    return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, GCAM, 0, LAYOUT>, grid, block, smem, st, p);
}

template <typename VT, bool MULTI, int LAYOUT>
static cudaError_t bwd_quad_flags(const MarchParams& p, bool gvol, bool gcam, int skip, unsigned grid,
                                  unsigned block, size_t smem, cudaStream_t st) {
    if (gvol && gcam)
        return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, true, 0, LAYOUT>, grid, block, smem, st, p);
    if (gvol) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, false, 0, LAYOUT>, grid, block, smem, st, p);
    if (gcam) return bwd_quad_skip<VT, MULTI, true, LAYOUT>(p, skip, grid, block, smem, st);
    return bwd_quad_skip<VT, MULTI, false, LAYOUT>(p, skip, grid, block, smem, st);
}

template <typename VT>
static cudaError_t bwd_quad_multi(const MarchParams& p, bool multi, bool gvol, bool gcam, int skip, bool labeled,
                                  unsigned grid, unsigned block, size_t smem, cudaStream_t st) {
    if constexpr (!std::is_same<VT, float>::value) {
        if (labeled) {
            if (!multi) return cudaErrorInvalidValue;
            return bwd_quad_flags<VT, true, kLayoutQuadLab>(p, gvol, gcam, skip, grid, block, smem, st);
        }
    } else {
        if (labeled) return cudaErrorInvalidValue;
    }
    return multi ? bwd_quad_flags<VT, true, kLayoutQuad>(p, gvol, gcam, skip, grid, block, smem, st)
                 : bwd_quad_flags<VT, false, kLayoutQuad>(p, gvol, gcam, skip, grid, block, smem, st);
}

cudaError_t launch_bwd_quad(const MarchParams& p, int vol_dtype, bool multi, bool gvol, bool gcam, int skip,
                            bool labeled, unsigned grid, unsigned block, size_t smem, cudaStream_t st) {
    switch (vol_dtype) {
        case NDRR_F32: return bwd_quad_multi<float>(p, multi, gvol, gcam, skip, labeled, grid, block, smem, st);
        case NDRR_F16: return bwd_quad_multi<__half>(p, multi, gvol, gcam, skip, labeled, grid, block, smem, st);
        case NDRR_BF16:
            return bwd_quad_multi<__nv_bfloat16>(p, multi, gvol, gcam, skip, labeled, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ndrr
