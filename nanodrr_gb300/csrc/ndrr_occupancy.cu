// Empty-space structures for the proposal-guided march.
//
// 1. Occupancy / distance grid. The volume is covered by cells of `cell`^3
//    voxels plus a one-cell border on every side; grid cell g (per axis) spans
//    voxels [(g - 1) * cell, g * cell). A cell is occupied when any voxel
//    within two voxels of it is non-zero: a sample whose floor position lies in
//    an unoccupied cell therefore has eight zero corners even if its position
//    is off by up to a voxel, so it contributes exactly nothing to the image,
//    the pose gradient or the camera gradients. The grid stores the Chebyshev
//    distance (in cells) to the nearest occupied cell, 0 for occupied cells,
//    capped at `max_dist`.
// 2. Extent labels. For every ray, the first and last sample of the box-culled
//    march whose eight corners are not all zero, as t = s / (S - 1) — the
//    non-empty interval the plain renderer itself sees (training labels for the
//    learned proposal).
#include <algorithm>

#include "ndrr_device.cuh"
#include "ndrr_launch.h"

namespace ndrr {

// ---------------------------------------------------------------- occupancy
template <typename VT>
__global__ void occupancy_kernel(const VT* __restrict__ vol, int D, int H, int W, int cell, int gx, int gy, int gz,
                                 uint8_t* __restrict__ dist, int max_dist) {
    const long long ncell = (long long)gx * gy * gz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncell;
         i += (long long)gridDim.x * blockDim.x) {
        const int cx = (int)(i % gx);
        const int cy = (int)((i / gx) % gy);
        const int cz = (int)(i / ((long long)gx * gy));
        const int x0 = max((cx - 1) * cell - 2, 0), x1 = min(cx * cell + 1, W - 1);
        const int y0 = max((cy - 1) * cell - 2, 0), y1 = min(cy * cell + 1, H - 1);
        const int z0 = max((cz - 1) * cell - 2, 0), z1 = min(cz * cell + 1, D - 1);
        bool occ = false;
        for (int z = z0; z <= z1 && !occ; ++z)
            for (int y = y0; y <= y1 && !occ; ++y) {
                const VT* row = vol + ((size_t)z * H + y) * W;
                for (int x = x0; x <= x1; ++x) {
                    if (ld_vox(row, x) != 0.f) {
                        occ = true;
                        break;
                    }
                }
            }
        dist[i] = occ ? 0 : (uint8_t)max_dist;
    }
}

// One pass of the Chebyshev distance transform: d = min(d, min over the 26
// neighbours + 1). After k passes every distance <= k is exact.
__global__ void distance_pass_kernel(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int gx, int gy,
                                     int gz) {
    const long long ncell = (long long)gx * gy * gz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncell;
         i += (long long)gridDim.x * blockDim.x) {
        const int cx = (int)(i % gx);
        const int cy = (int)((i / gx) % gy);
        const int cz = (int)(i / ((long long)gx * gy));
        int d = src[i];
        if (d > 0) {
            for (int dz = -1; dz <= 1; ++dz) {
                const int z = cz + dz;
                if (z < 0 || z >= gz) continue;
                for (int dy = -1; dy <= 1; ++dy) {
                    const int y = cy + dy;
                    if (y < 0 || y >= gy) continue;
                    const uint8_t* row = src + ((size_t)z * gy + y) * gx;
                    for (int dx = -1; dx <= 1; ++dx) {
                        const int x = cx + dx;
                        if (x < 0 || x >= gx) continue;
                        d = min(d, (int)row[x] + 1);
                    }
                }
            }
        }
        dst[i] = (uint8_t)d;
    }
}

cudaError_t launch_occupancy(const void* vol, int vol_dtype, int D, int H, int W, int cell, int max_dist,
                             uint8_t* dist, uint8_t* scratch, cudaStream_t st) {
    const int gx = (W + cell - 1) / cell + 2, gy = (H + cell - 1) / cell + 2, gz = (D + cell - 1) / cell + 2;
    const long long ncell = (long long)gx * gy * gz;
    const int block = 256;
    const int grid = (int)std::min<long long>((ncell + block - 1) / block, 152LL * 32);
    switch (vol_dtype) {
        case NDRR_F32:
            occupancy_kernel<<<grid, block, 0, st>>>((const float*)vol, D, H, W, cell, gx, gy, gz, dist, max_dist);
            break;
        case NDRR_F16:
            occupancy_kernel<<<grid, block, 0, st>>>((const __half*)vol, D, H, W, cell, gx, gy, gz, dist, max_dist);
            break;
        case NDRR_BF16:
            occupancy_kernel<<<grid, block, 0, st>>>((const __nv_bfloat16*)vol, D, H, W, cell, gx, gy, gz, dist,
                                                     max_dist);
            break;
        default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // Ping-pong so that the final distances land in `dist`.
    uint8_t* a = dist;
    uint8_t* b = scratch;
    for (int k = 0; k < max_dist; ++k) {
        distance_pass_kernel<<<grid, block, 0, st>>>(a, b, gx, gy, gz);
        std::swap(a, b);
    }
    if (a != dist) cudaMemcpyAsync(dist, a, (size_t)ncell, cudaMemcpyDeviceToDevice, st);
    return cudaGetLastError();
}

}  // namespace ndrr
