// Internal launch interface between the C ABI (ndrr_capi.cu) and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nanodrr_gb300.h"

namespace ndrr {

struct LaunchShape {
    int tw = 16;  // tile width in rays (multiple of 8)
    int th = 8;   // tile height in rays (multiple of 4)
    int K = 1;    // sample chunks per ray within a CTA
    bool brick = false;  // adjoint: per-slab shared-memory volume-gradient brick
    int cap = 0;         // brick capacity in voxels
    int L0 = 16;         // initial slab length in samples
    int sm = 0;          // SM count of the device (0 when unknown)
    bool slab = false;   // adjoint with volume gradient ordered slab by slab (quad layout)
    bool split = false;  // slab: pose pass with gathers, then a positions-only scatter pass
};

// Measurement hook (ndrr_set_kernel_events): CUDA events recorded on the
// launch stream just before and just after each ray-march kernel launch of
// the calling thread; NULL when off.
struct KernelEvents {
    cudaEvent_t start = nullptr;
    cudaEvent_t stop = nullptr;
};
KernelEvents& kernel_events();
cudaError_t launch_l2_probe(const void* buf, unsigned long long bytes, int passes, unsigned* sink, int sm_count,
                            cudaStream_t st);
cudaError_t launch_reduce_probe(void* buf, int planes, int iters, int sm_count, cudaStream_t st);

LaunchShape choose_shape(const ndrr_raymarch_args& a, int sm_count);
uint64_t bwd_workspace_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);
size_t fwd_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);
size_t bwd_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);
size_t bwd_epilogue_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);
size_t brick_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);

cudaError_t launch_fwd(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st);
cudaError_t launch_skip_windows(const ndrr_raymarch_args& a, int32_t* windows, cudaStream_t st);
cudaError_t launch_fwd_tex(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st);
cudaError_t launch_fwd_tma(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st);
cudaError_t texture_create(const float* vol, int D, int H, int W, unsigned long long* handle, cudaStream_t st);
cudaError_t texture_destroy(unsigned long long handle, bool* known);
cudaError_t launch_bwd(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st);
uint64_t slab_workspace_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);
float* slab_partials(const ndrr_raymarch_args& a, const LaunchShape& ls);
int homography_blocks(int H, int W);
size_t ncc_workspace_bytes(int B, int P, int N);
cudaError_t launch_ncc_fwd(const float* x1, const float* x2, int B, int P, int N, float eps, float* score,
                           float* stats, void* workspace, cudaStream_t st);
cudaError_t launch_ncc_bwd(const float* go, const float* x1, const float* x2, const float* stats, int B, int P,
                           int N, float* g1, float* g2, cudaStream_t st);
cudaError_t launch_pose_fwd(const float* rot, const float* xyz, int param_rows, const float* rt_inv,
                            const float* pivot, const float* pivot_inv, int B, float* pose, cudaStream_t st);
cudaError_t launch_pose_bwd(const float* gpose, const float* rot, const float* xyz, int param_rows,
                            const float* rt_inv, const float* pivot, const float* pivot_inv, int B, float* g_rot,
                            float* g_xyz, cudaStream_t st);
cudaError_t launch_homography_fwd(const float* img, const float* hom, int B, int C, int H, int W, float* out,
                                  cudaStream_t st);
cudaError_t launch_homography_bwd(const float* go, const float* img, const float* hom, int B, int C, int H, int W,
                                  float* gimg, float* ghom, float* partials, cudaStream_t st);
cudaError_t launch_batched(const ndrr_batch_args& a, bool backward, int sm_count, cudaStream_t st);
cudaError_t device_flags(unsigned* out, bool clear);
cudaError_t launch_camera_rays(const float* k_inv, int n_k, const float* sdd, int n_s, int B, int height, int width,
                               int orthographic, float* src, float* tgt, cudaStream_t st);
cudaError_t launch_hu_to_mu(const void* hu, int dtype, long long n, float mu_water, float dmu, float hu_bone,
                            void* mu, cudaStream_t st);
cudaError_t launch_occupancy(const void* vol, int vol_dtype, int D, int H, int W, int cell, int max_dist,
                             uint8_t* dist, uint8_t* scratch, cudaStream_t st);

}  // namespace ndrr
