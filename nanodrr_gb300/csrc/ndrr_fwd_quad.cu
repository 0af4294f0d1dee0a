// Forward instantiations for the quad volume layouts (output in the volume's
// dtype, every skip mode): the quad layout for every volume dtype, and the
// labelled quad layout for 16-bit volumes with label channels.
#include <type_traits>

#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT, bool MULTI, int LAYOUT>
static cudaError_t fwd_quad_skip(const MarchParams& p, int skip, unsigned grid, unsigned block, size_t smem,
                                 cudaStream_t st) {
    if (skip == NDRR_SKIP_OCCUPANCY)
        return launch_kernel(raymarch_fwd_kernel<VT, VT, MULTI, 1, LAYOUT>, grid, block, smem, st, p);
    return launch_kernel(raymarch_fwd_kernel<VT, VT, MULTI, 0, LAYOUT>, grid, block, smem, st, p);
}

template <typename VT>
static cudaError_t fwd_quad_multi(const MarchParams& p, bool multi, int skip, bool labeled, unsigned grid,
                                  unsigned block, size_t smem, cudaStream_t st) {
    if constexpr (!std::is_same<VT, float>::value) {
        if (labeled) {
            if (!multi) return cudaErrorInvalidValue;
            return fwd_quad_skip<VT, true, kLayoutQuadLab>(p, skip, grid, block, smem, st);
        }
    } else {
        if (labeled) return cudaErrorInvalidValue;
    }
    return multi ? fwd_quad_skip<VT, true, kLayoutQuad>(p, skip, grid, block, smem, st)
                 : fwd_quad_skip<VT, false, kLayoutQuad>(p, skip, grid, block, smem, st);
}

cudaError_t launch_fwd_quad(const MarchParams& p, int vol_dtype, bool multi, int skip, bool labeled, unsigned grid,
                            unsigned block, size_t smem, cudaStream_t st) {
    switch (vol_dtype) {
        case NDRR_F32: return fwd_quad_multi<float>(p, multi, skip, labeled, grid, block, smem, st);
        case NDRR_F16: return fwd_quad_multi<__half>(p, multi, skip, labeled, grid, block, smem, st);
        case NDRR_BF16: return fwd_quad_multi<__nv_bfloat16>(p, multi, skip, labeled, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ndrr
