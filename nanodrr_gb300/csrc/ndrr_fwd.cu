// Forward launcher: instantiates the forward kernel for each volume dtype,
// output dtype, label mode and skip mode (skip modes only with the output in
// the volume's dtype, the render call's case).
#include <type_traits>

#include "ndrr_march.cuh"

namespace ndrr {

template <typename VT, typename OT, bool MULTI>
static cudaError_t fwd_dispatch_skip(const MarchParams& p, int skip, unsigned grid, unsigned block, size_t smem,
                                     cudaStream_t st) {
    if constexpr (std::is_same<VT, OT>::value) {
        if (skip == NDRR_SKIP_OCCUPANCY)
            return launch_kernel(raymarch_fwd_kernel<VT, OT, MULTI, 1, kLayoutVolume>, grid, block, smem, st, p);
    } else {
        if (skip != NDRR_SKIP_NONE) return cudaErrorNotSupported;
    }
    return launch_kernel(raymarch_fwd_kernel<VT, OT, MULTI, 0, kLayoutVolume>, grid, block, smem, st, p);
}

template <typename VT, typename OT>
static cudaError_t fwd_dispatch_multi(const MarchParams& p, bool multi, int skip, unsigned grid, unsigned block,
                                      size_t smem, cudaStream_t st) {
    if (multi) return fwd_dispatch_skip<VT, OT, true>(p, skip, grid, block, smem, st);
    return fwd_dispatch_skip<VT, OT, false>(p, skip, grid, block, smem, st);
}

template <typename VT>
static cudaError_t fwd_dispatch_out(const MarchParams& p, int out_dtype, bool multi, int skip, unsigned grid,
                                    unsigned block, size_t smem, cudaStream_t st) {
    switch (out_dtype) {
        case NDRR_F32: return fwd_dispatch_multi<VT, float>(p, multi, skip, grid, block, smem, st);
        case NDRR_F16: return fwd_dispatch_multi<VT, __half>(p, multi, skip, grid, block, smem, st);
        case NDRR_BF16: return fwd_dispatch_multi<VT, __nv_bfloat16>(p, multi, skip, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fwd(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st) {
    MarchParams p = make_params(a, ls);
    unsigned grid = (unsigned)((size_t)a.B * p.tm.tiles);
    const unsigned block = (unsigned)(ls.tw * ls.th * ls.K);
    const size_t smem = fwd_smem_bytes(a, ls);
    const bool multi = a.n_classes > 1;
    const int skip = a.skip_mode;
    if (a.vol_quad != nullptr) {
        if (a.out_dtype != a.vol_dtype) return cudaErrorNotSupported;
        return launch_fwd_quad(p, a.vol_dtype, multi, skip, a.quad_labels != 0, grid, block, smem, st);
    }
    switch (a.vol_dtype) {
        case NDRR_F32: return fwd_dispatch_out<float>(p, a.out_dtype, multi, skip, grid, block, smem, st);
        case NDRR_F16: return fwd_dispatch_out<__half>(p, a.out_dtype, multi, skip, grid, block, smem, st);
        case NDRR_BF16: return fwd_dispatch_out<__nv_bfloat16>(p, a.out_dtype, multi, skip, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace ndrr
