// Distance-field traversal of the occupancy grid built by ndrr_occupancy.cu.
//
// Grid cell g (per axis) spans voxels [(g - 1) * cell, g * cell); its value is
// the Chebyshev distance in cells to the nearest occupied cell (0: occupied).
// A value d > 0 means the (2d - 1)^3 cube of cells centred on g is empty, so a
// ray can jump to the exit of that cube in one step. Positions outside the
// grid lie more than a cell away from every voxel and are empty.
#pragma once

#include "ndrr_device.cuh"

namespace ndrr {

struct OccGrid {
    const uint8_t* __restrict__ dist;
    int gx, gy, gz;
    int cell;
};

// Ray-parameter interval where the position lies inside the grid box.
__device__ __forceinline__ bool grid_interval(const OccGrid& g, const Ray& r, float& t0, float& t1) {
    const float c = (float)g.cell;
    float a0, a1, b0, b1, c0, c1;
    axis_interval(r.p0x, r.dx, -c, (float)(g.gx - 1) * c, a0, a1);
    axis_interval(r.p0y, r.dy, -c, (float)(g.gy - 1) * c, b0, b1);
    axis_interval(r.p0z, r.dz, -c, (float)(g.gz - 1) * c, c0, c1);
    t0 = fmaxf(fmaxf(a0, b0), c0);
    t1 = fminf(fminf(a1, b1), c1);
    return t0 <= t1;
}

// Parameter at which the ray, currently inside the voxel box [lo, hi) on every
// axis, leaves it (the nearest exit face in the direction of travel).
__device__ __forceinline__ float box_exit(const Ray& r, float t, float lox, float hix, float loy, float hiy,
                                          float loz, float hiz) {
    float te = INFINITY;
    if (r.dx > 0.f) te = fminf(te, (hix - r.p0x) / r.dx);
    if (r.dx < 0.f) te = fminf(te, (lox - r.p0x) / r.dx);
    if (r.dy > 0.f) te = fminf(te, (hiy - r.p0y) / r.dy);
    if (r.dy < 0.f) te = fminf(te, (loy - r.p0y) / r.dy);
    if (r.dz > 0.f) te = fminf(te, (hiz - r.p0z) / r.dz);
    if (r.dz < 0.f) te = fminf(te, (loz - r.p0z) / r.dz);
    return fmaxf(te, t);
}

// March the distance field from ta toward tb (tb < ta marches backward).
// Returns 1 when an occupied cell is met (its parameter in *t_hit), 0 when
// the whole segment is empty, -1 when the step budget ran out (unknown:
// callers treat it as occupied, which is conservative).
__device__ __forceinline__ int first_occupied(const OccGrid& g, Ray r, float ta, float tb, int max_steps,
                                              float* t_hit) {
    // March backward by flipping the ray: u = -t.
    const bool back = tb < ta;
    if (back) {
        r.dx = -r.dx;
        r.dy = -r.dy;
        r.dz = -r.dz;
        ta = -ta;
        tb = -tb;
    }
    float g0, g1;
    if (!grid_interval(g, r, g0, g1)) return 0;
    float t = fmaxf(ta, g0);
    const float tend = fminf(tb, g1);
    if (t > tend) return 0;
    const float c = (float)g.cell, inv_c = 1.0f / c;
    const float dmax = fmaxf(fmaxf(fabsf(r.dx), fabsf(r.dy)), fabsf(r.dz));
    const float eps = dmax > 0.f ? 1e-3f / dmax : 1e30f;  // a thousandth of a voxel
    for (int it = 0; it < max_steps; ++it) {
        if (t > tend) return 0;
        const float px = fmaf(t, r.dx, r.p0x), py = fmaf(t, r.dy, r.p0y), pz = fmaf(t, r.dz, r.p0z);
        const int cx = min(max((int)floorf(px * inv_c) + 1, 0), g.gx - 1);
        const int cy = min(max((int)floorf(py * inv_c) + 1, 0), g.gy - 1);
        const int cz = min(max((int)floorf(pz * inv_c) + 1, 0), g.gz - 1);
        const int d = __ldg(g.dist + ((size_t)cz * g.gy + cy) * g.gx + cx);
        if (d == 0) {
            *t_hit = back ? -t : t;
            return 1;
        }
        // Empty cube of cells [c - d + 1, c + d - 1] -> voxels [(c - d) cell, (c + d - 1) cell).
        const float lox = (float)(cx - d) * c, hix = (float)(cx + d - 1) * c;
        const float loy = (float)(cy - d) * c, hiy = (float)(cy + d - 1) * c;
        const float loz = (float)(cz - d) * c, hiz = (float)(cz + d - 1) * c;
        t = box_exit(r, t, lox, hix, loy, hiy, loz, hiz) + eps;
    }
    return -1;
}

}  // namespace ndrr
