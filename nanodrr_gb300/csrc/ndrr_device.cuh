// Device-side helpers shared by the ray-march kernels: element loads, the
// per-ray set-up (camera -> voxel line and sample window) and the trilinear
// sample with zero padding.
//
// Sampling semantics follow the reference's fused kernel (nanodrr
// src/nanodrr/drr/_fused.py:133-228), which in turn reproduces grid_sample
// (bilinear, zeros padding, align_corners=False) in voxel-index coordinates:
// sample s of a ray sits at p0 + t_s * d with t_s = s / (S - 1); out-of-range
// corners read as 0; labels use the nearest voxel with ties to even.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/nanodrr_gb300.h"

namespace ndrr {

// ---------------------------------------------------------------- element I/O
template <typename T>
__device__ __forceinline__ float ld_vox(const T* __restrict__ p, int idx);

template <>
__device__ __forceinline__ float ld_vox<float>(const float* __restrict__ p, int idx) {
    return __ldg(p + idx);
}
template <>
__device__ __forceinline__ float ld_vox<__half>(const __half* __restrict__ p, int idx) {
    return __half2float(__ldg(p + idx));
}
template <>
__device__ __forceinline__ float ld_vox<__nv_bfloat16>(const __nv_bfloat16* __restrict__ p, int idx) {
    return __bfloat162float(__ldg(p + idx));
}

template <typename T>
__device__ __forceinline__ void st_out(T* p, size_t idx, float v);
template <>
__device__ __forceinline__ void st_out<float>(float* p, size_t idx, float v) { p[idx] = v; }
template <>
__device__ __forceinline__ void st_out<__half>(__half* p, size_t idx, float v) { p[idx] = __float2half_rn(v); }
template <>
__device__ __forceinline__ void st_out<__nv_bfloat16>(__nv_bfloat16* p, size_t idx, float v) {
    p[idx] = __float2bfloat16_rn(v);
}

// Generic element read used for labels and upstream gradients, whose dtype is
// a runtime value (uniform across the launch, so the switch never diverges).
__device__ __forceinline__ float ld_any_f(const void* __restrict__ p, int dtype, size_t idx) {
    switch (dtype) {
        case NDRR_F32: return __ldg(reinterpret_cast<const float*>(p) + idx);
        case NDRR_F16: return __half2float(__ldg(reinterpret_cast<const __half*>(p) + idx));
        case NDRR_BF16: return __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p) + idx));
        default: return 0.f;
    }
}

// Label value -> class index. Float labels convert with truncation toward zero
// (a cast, as `.to(int32)` / `.long()` do in the reference, _fused.py:228 and
// backends.py:57). Values that do not fit in int32 map to -1 (dropped).
__device__ __forceinline__ int ld_label(const void* __restrict__ p, int dtype, int idx) {
    switch (dtype) {
        case NDRR_F32: {
            float v = __ldg(reinterpret_cast<const float*>(p) + idx);
            return (v > -2147483520.f && v < 2147483520.f) ? __float2int_rz(v) : -1;
        }
        case NDRR_F16: return __float2int_rz(__half2float(__ldg(reinterpret_cast<const __half*>(p) + idx)));
        case NDRR_BF16: {
            float v = __bfloat162float(__ldg(reinterpret_cast<const __nv_bfloat16*>(p) + idx));
            return (v > -2147483520.f && v < 2147483520.f) ? __float2int_rz(v) : -1;
        }
        case NDRR_U8: return (int)__ldg(reinterpret_cast<const uint8_t*>(p) + idx);
        case NDRR_I8: return (int)__ldg(reinterpret_cast<const int8_t*>(p) + idx);
        case NDRR_I16: return (int)__ldg(reinterpret_cast<const int16_t*>(p) + idx);
        case NDRR_I32: return __ldg(reinterpret_cast<const int*>(p) + idx);
        case NDRR_I64: {
            long long v = __ldg(reinterpret_cast<const long long*>(p) + idx);
            return (v >= -2147483647LL && v <= 2147483647LL) ? (int)v : -1;
        }
        default: return -1;
    }
}

// ------------------------------------------------------------------ geometry
struct Ray {
    float p0x, p0y, p0z;  // voxel-space position of the source (t = 0)
    float dx, dy, dz;     // voxel-space displacement src -> tgt
    int lo, hi;           // sample window [lo, hi): samples outside contribute 0
};

// Parameter interval where lo <= p + t * d <= hi along one axis.
__device__ __forceinline__ void axis_interval(float p, float d, float lo, float hi, float& t0, float& t1) {
    if (fabsf(d) < 1e-20f) {
        const bool inside = (p >= lo) && (p <= hi);
        t0 = inside ? -INFINITY : INFINITY;
        t1 = inside ? INFINITY : -INFINITY;
        return;
    }
    const float inv = 1.0f / d;
    const float a = (lo - p) * inv;
    const float b = (hi - p) * inv;
    t0 = fminf(a, b);
    t1 = fmaxf(a, b);
}

// Sample window of a ray: every sample whose trilinear footprint can touch the
// volume lies in [lo, hi). The box is the footprint support (-1, dim) widened
// by one voxel, and the index range is widened by -2/+3 samples, so rounding
// in this set-up can never drop a contributing sample (the same conservative
// rule as the reference's cull, _fused.py:144-155, applied per ray instead of
// per 128-ray program). Skipped samples contribute exactly zero to every
// output and gradient.
__device__ __forceinline__ void ray_window(Ray& r, int D, int H, int W, int S) {
    float ax0, ax1, ay0, ay1, az0, az1;
    axis_interval(r.p0x, r.dx, -2.0f, (float)W + 1.0f, ax0, ax1);
    axis_interval(r.p0y, r.dy, -2.0f, (float)H + 1.0f, ay0, ay1);
    axis_interval(r.p0z, r.dz, -2.0f, (float)D + 1.0f, az0, az1);
    const float t_lo = fmaxf(fmaxf(ax0, ay0), az0);
    const float t_hi = fminf(fminf(ax1, ay1), az1);
    const float sm1 = (float)(S - 1);
    if (!(t_lo <= t_hi)) {
        r.lo = 0;
        r.hi = 0;
        return;
    }
    // Clamp before converting so huge or infinite parameters stay in range.
    const float f_lo = fminf(fmaxf(floorf(t_lo * sm1) - 2.0f, 0.0f), (float)S);
    const float f_hi = fminf(fmaxf(ceilf(t_hi * sm1) + 3.0f, 0.0f), (float)S);
    r.lo = (int)f_lo;
    r.hi = (int)f_hi;
}

// Intersect the window with an optional per-ray [t_lo, t_hi] (in units of t).
__device__ __forceinline__ void apply_t_window(Ray& r, float wlo, float whi, int S) {
    const float sm1 = (float)(S - 1);
    const float a = fminf(fmaxf(ceilf(wlo * sm1), 0.0f), (float)S);
    const float b = fminf(fmaxf(floorf(whi * sm1) + 1.0f, 0.0f), (float)S);
    r.lo = max(r.lo, (int)a);
    r.hi = min(r.hi, (int)b);
}

// ------------------------------------------------- fixed-point ray positions
// A sample's position p0 + s * step (voxel index space) is carried in 32.32
// fixed point: int64 counts of 2^-32 voxel. The cell is the integer part and
// the trilinear weights come from the fractional part, so a position keeps
// 2^-32 voxel resolution anywhere in the volume, where a float keeps 2^-9 at
// 512 (ulp 6.1e-5 voxel). This matters for the gradients: the trilinear
// derivative jumps at every cell face, and float positions put about one
// sample in 10^4 on the other side of a face than the exact (float64)
// position does, which moves pose gradients at the 1e-3 level. The start p0
// and the step are formed per ray in float-float arithmetic (error-free
// products and sums on fp32, about 44 significant bits) from the inputs, so
// positions match the float64 oracle's to ~2e-7 voxel after 800 samples.
struct FixPos {
    long long x, y, z;
};

__device__ __forceinline__ int fix_floor(long long v) { return (int)(v >> 32); }

// The top 23 bits of the fraction, exactly, as a float in [0, 1).
__device__ __forceinline__ float fix_frac(long long v) {
    return __int_as_float(0x3f800000u | ((unsigned)v >> 9)) - 1.0f;
}

// Nearest integer, ties to even (the nearest-label rule), on the exact value.
__device__ __forceinline__ int fix_round(long long v) {
    const int f = fix_floor(v);
    const unsigned lo = (unsigned)v;
    return f + ((lo > 0x80000000u) || (lo == 0x80000000u && (f & 1)) ? 1 : 0);
}

__device__ __forceinline__ FixPos fix_add(const FixPos& a, const FixPos& b) {
    return FixPos{a.x + b.x, a.y + b.y, a.z + b.z};
}

// Float-float helpers (value = hi + lo) for the per-ray set-up, written with
// _rn intrinsics so the compiler cannot contract or reorder them.
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 f2_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return F2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ F2 f2_norm(float hi, float lo) {
    const float s = __fadd_rn(hi, lo);
    return F2{s, __fsub_rn(lo, __fsub_rn(s, hi))};
}

__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const F2 s = f2_two_sum(a.hi, b.hi);
    return f2_norm(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);  // exact error of the product
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return f2_norm(p, e);
}

// a / n for an integer n exactly representable in fp32: the remainder of the
// leading quotient is exact with an FMA.
__device__ __forceinline__ F2 f2_div_int(F2 a, float n) {
    const float q = __fdiv_rn(a.hi, n);
    const float r = __fmaf_rn(-q, n, a.hi);
    return f2_norm(q, __fdiv_rn(__fadd_rn(r, a.lo), n));
}

// float-float -> 32.32 fixed point, clamped to +-2^30 voxels (a ray that far
// out has an empty window anyway); hi * 2^32 and lo * 2^32 are exact scalings.
__device__ __forceinline__ long long f2_to_fix(F2 v) {
    const float hi = fminf(fmaxf(v.hi, -1073741824.0f), 1073741824.0f);
    const float lo = hi == v.hi ? v.lo : 0.0f;
    return __float2ll_rn(__fmul_rn(hi, 4294967296.0f)) + __float2ll_rn(__fmul_rn(lo, 4294967296.0f));
}

// ------------------------------------------------------------ trilinear tap
// The eight corners of the cell containing (x, y, z), zero outside the volume,
// and the fractional offsets inside the cell.
struct Cell {
    float v000, v001, v010, v011, v100, v101, v110, v111;  // v[z][y][x] offsets
    float fx, fy, fz;
    int ix, iy, iz;
    int cls;  // labelled quad layout only: class of the nearest corner (255 = dropped)
};

// ------------------------------------------------------------ quad layout
// A padded copy of the volume in which element (qz, qy, qx) holds the four
// corners (x0, y0), (x0 + 1, y0), (x0, y0 + 1), (x0 + 1, y0 + 1) of plane
// z = qz - 2, with x0 = qx - 2 and y0 = qy - 2, zeros outside the volume.
// Extent: QX = W + 3, QY = H + 3, QZ = D + 4 (cells with x0 in [-2, W],
// y0 in [-2, H], both planes of z0 in [-2, D]). A sample then needs two
// vector loads (planes z0 and z0 + 1) and no bounds checks: any position is
// clamped into the zero border, where all corners are 0.
template <typename VT>
struct QuadOf;
template <>
struct QuadOf<float> {
    using T = float4;
};
template <>
struct QuadOf<__half> {
    using T = uint2;
};
template <>
struct QuadOf<__nv_bfloat16> {
    using T = uint2;
};

struct QuadGeom {
    int qx, qy;      // padded row length and rows per plane
    int plane;       // qx * qy
};

__host__ __device__ __forceinline__ QuadGeom make_quadgeom(int D, int H, int W) {
    (void)D;
    QuadGeom g;
    g.qx = W + 3;
    g.qy = H + 3;
    g.plane = g.qx * g.qy;
    return g;
}

__device__ __forceinline__ void unpack_quad(float4 q, float& a, float& b, float& c, float& d) {
    a = q.x;
    b = q.y;
    c = q.z;
    d = q.w;
}

// bf16 -> f32 is exact: a bf16 value is the high half of the f32 bit pattern.
__device__ __forceinline__ void unpack_quad_bf16(uint2 q, float& a, float& b, float& c, float& d) {
    a = __uint_as_float(q.x << 16);
    b = __uint_as_float(q.x & 0xffff0000u);
    c = __uint_as_float(q.y << 16);
    d = __uint_as_float(q.y & 0xffff0000u);
}

__device__ __forceinline__ void unpack_quad_f16(uint2 q, float& a, float& b, float& c, float& d) {
    const __half2 h0 = *reinterpret_cast<const __half2*>(&q.x);
    const __half2 h1 = *reinterpret_cast<const __half2*>(&q.y);
    const float2 f0 = __half22float2(h0), f1 = __half22float2(h1);
    a = f0.x;
    b = f0.y;
    c = f1.x;
    d = f1.y;
}

__device__ __forceinline__ float cell_value(const Cell& c) {
    const float c00 = fmaf(c.fx, c.v001 - c.v000, c.v000);
    const float c01 = fmaf(c.fx, c.v011 - c.v010, c.v010);
    const float c10 = fmaf(c.fx, c.v101 - c.v100, c.v100);
    const float c11 = fmaf(c.fx, c.v111 - c.v110, c.v110);
    const float c0 = fmaf(c.fy, c01 - c00, c00);
    const float c1 = fmaf(c.fy, c11 - c10, c10);
    return fmaf(c.fz, c1 - c0, c0);
}

// Analytic derivative of the trilinear interpolant with respect to the
// voxel-space position (the partial derivatives of the formula above).
// Written with explicit fmaf so every kernel instantiation rounds the same
// way (the compiler would otherwise be free to contract differently).
__device__ __forceinline__ void cell_grad(const Cell& c, float& gx, float& gy, float& gz) {
    const float wx0 = 1.f - c.fx, wy0 = 1.f - c.fy, wz0 = 1.f - c.fz;
    const float x00 = fmaf(c.v011 - c.v010, c.fy, __fmul_rn(c.v001 - c.v000, wy0));
    const float x11 = fmaf(c.v111 - c.v110, c.fy, __fmul_rn(c.v101 - c.v100, wy0));
    gx = fmaf(x11, c.fz, __fmul_rn(x00, wz0));
    const float y00 = fmaf(c.v011 - c.v001, c.fx, __fmul_rn(c.v010 - c.v000, wx0));
    const float y11 = fmaf(c.v111 - c.v101, c.fx, __fmul_rn(c.v110 - c.v100, wx0));
    gy = fmaf(y11, c.fz, __fmul_rn(y00, wz0));
    const float z00 = fmaf(c.v101 - c.v001, c.fx, __fmul_rn(c.v100 - c.v000, wx0));
    const float z11 = fmaf(c.v111 - c.v011, c.fx, __fmul_rn(c.v110 - c.v010, wx0));
    gz = fmaf(z11, c.fy, __fmul_rn(z00, wy0));
}

// ---------------------------------------------- float positions (forward)
// The forward evaluates sample positions in float32, as p0 + t * d with one
// rounding (its images are within 1e-6 of the float64 oracle at 512^3); the
// adjoint, whose gradients jump at cell faces, uses the fixed-point versions
// below. Positions are clamped to [-2, dim + 1] first: beyond that every
// corner is outside the volume either way, and the clamp keeps the float ->
// int conversion in range for any input.
template <typename VT>
__device__ __forceinline__ void load_cell(const VT* __restrict__ vol, int D, int H, int W, float x, float y,
                                          float z, Cell& c) {
    // Positions are clamped to [-2, dim + 1] first: beyond that every corner
    // is outside the volume either way, and the clamp keeps the float -> int
    // conversion in range for any input.
    x = fminf(fmaxf(x, -2.0f), (float)W + 1.0f);
    y = fminf(fmaxf(y, -2.0f), (float)H + 1.0f);
    z = fminf(fmaxf(z, -2.0f), (float)D + 1.0f);
    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
    c.fx = x - xf;
    c.fy = y - yf;
    c.fz = z - zf;
    const int ix = (int)xf, iy = (int)yf, iz = (int)zf;
    c.ix = ix;
    c.iy = iy;
    c.iz = iz;
    const int HW = H * W;
    const int base = (iz * H + iy) * W + ix;
    if ((unsigned)ix < (unsigned)(W - 1) && (unsigned)iy < (unsigned)(H - 1) && (unsigned)iz < (unsigned)(D - 1)) {
        c.v000 = ld_vox(vol, base);
        c.v001 = ld_vox(vol, base + 1);
        c.v010 = ld_vox(vol, base + W);
        c.v011 = ld_vox(vol, base + W + 1);
        c.v100 = ld_vox(vol, base + HW);
        c.v101 = ld_vox(vol, base + HW + 1);
        c.v110 = ld_vox(vol, base + HW + W);
        c.v111 = ld_vox(vol, base + HW + W + 1);
    } else {
        const bool x0 = (unsigned)ix < (unsigned)W, x1 = (unsigned)(ix + 1) < (unsigned)W;
        const bool y0 = (unsigned)iy < (unsigned)H, y1 = (unsigned)(iy + 1) < (unsigned)H;
        const bool z0 = (unsigned)iz < (unsigned)D, z1 = (unsigned)(iz + 1) < (unsigned)D;
        c.v000 = (z0 && y0 && x0) ? ld_vox(vol, base) : 0.f;
        c.v001 = (z0 && y0 && x1) ? ld_vox(vol, base + 1) : 0.f;
        c.v010 = (z0 && y1 && x0) ? ld_vox(vol, base + W) : 0.f;
        c.v011 = (z0 && y1 && x1) ? ld_vox(vol, base + W + 1) : 0.f;
        c.v100 = (z1 && y0 && x0) ? ld_vox(vol, base + HW) : 0.f;
        c.v101 = (z1 && y0 && x1) ? ld_vox(vol, base + HW + 1) : 0.f;
        c.v110 = (z1 && y1 && x0) ? ld_vox(vol, base + HW + W) : 0.f;
        c.v111 = (z1 && y1 && x1) ? ld_vox(vol, base + HW + W + 1) : 0.f;
    }
}

// Quad index of the cell whose lower corner is the floor of (x, y, z),
// clamped into the padded extent, plus the fractional offsets and the cell's
// (clamped) corner indices for the gradient scatter.
__device__ __forceinline__ int quad_cell(const QuadGeom& g, int D, int H, int W, float x, float y, float z,
                                         Cell& c) {
    x = fminf(fmaxf(x, -2.0f), (float)W + 1.0f);
    y = fminf(fmaxf(y, -2.0f), (float)H + 1.0f);
    z = fminf(fmaxf(z, -2.0f), (float)D + 1.0f);
    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
    c.fx = x - xf;
    c.fy = y - yf;
    c.fz = z - zf;
    c.ix = min((int)xf, W);
    c.iy = min((int)yf, H);
    c.iz = min((int)zf, D);
    return ((c.iz + 2) * g.qy + (c.iy + 2)) * g.qx + (c.ix + 2);
}

template <typename VT>
__device__ __forceinline__ void load_cell_quad(const void* __restrict__ quad, const QuadGeom& g, int D, int H,
                                               int W, float x, float y, float z, Cell& c) {
    const int qi = quad_cell(g, D, H, W, x, y, z, c);
    using Q = typename QuadOf<VT>::T;
    const Q* __restrict__ qp = reinterpret_cast<const Q*>(quad);
    const Q q0 = __ldg(qp + qi);
    const Q q1 = __ldg(qp + qi + g.plane);
    if constexpr (std::is_same<VT, float>::value) {
        unpack_quad(q0, c.v000, c.v001, c.v010, c.v011);
        unpack_quad(q1, c.v100, c.v101, c.v110, c.v111);
    } else if constexpr (std::is_same<VT, __nv_bfloat16>::value) {
        unpack_quad_bf16(q0, c.v000, c.v001, c.v010, c.v011);
        unpack_quad_bf16(q1, c.v100, c.v101, c.v110, c.v111);
    } else {
        unpack_quad_f16(q0, c.v000, c.v001, c.v010, c.v011);
        unpack_quad_f16(q1, c.v100, c.v101, c.v110, c.v111);
    }
}

// Labelled quad at a float position (see load_cell_quad_labeled_fix).
template <typename VT>
__device__ __forceinline__ void load_cell_quad_labeled(const void* __restrict__ quad, const QuadGeom& g, int D, int H,
                                                       int W, float x, float y, float z, Cell& c) {
    const int qi = quad_cell(g, D, H, W, x, y, z, c);
    const uint4* __restrict__ qp = reinterpret_cast<const uint4*>(quad);
    const uint4 q0 = __ldg(qp + qi);
    const uint4 q1 = __ldg(qp + qi + g.plane);
    if constexpr (std::is_same<VT, __nv_bfloat16>::value) {
        unpack_quad_bf16(make_uint2(q0.x, q0.y), c.v000, c.v001, c.v010, c.v011);
        unpack_quad_bf16(make_uint2(q1.x, q1.y), c.v100, c.v101, c.v110, c.v111);
    } else {
        unpack_quad_f16(make_uint2(q0.x, q0.y), c.v000, c.v001, c.v010, c.v011);
        unpack_quad_f16(make_uint2(q1.x, q1.y), c.v100, c.v101, c.v110, c.v111);
    }
    // Nearest corner, ties to even: rint of the clamped coordinate minus the
    // cell's corner, read from the fraction quad_cell already formed (1 past
    // one half, or at one half on an odd corner). Where the clamp moved the
    // cell every corner lies outside the volume and carries class 0, so the
    // choice there cannot change the class.
    const int ox = (c.fx > 0.5f) | ((c.fx == 0.5f) & (c.ix & 1));
    const int oy = (c.fy > 0.5f) | ((c.fy == 0.5f) & (c.iy & 1));
    const int oz = (c.fz > 0.5f) | ((c.fz == 0.5f) & (c.iz & 1));
    // byte ox + 2 oy of plane oz's class word: one byte permute over both
    c.cls = (int)(__byte_perm(q0.z, q1.z, (unsigned)(ox + 2 * oy + 4 * oz)) & 0xffu);
}

// Nearest-voxel label at (x, y, z); ties round to even like grid_sample's
// nearest mode. Out-of-volume positions read label 0 (zero padding).
__device__ __forceinline__ int nearest_label(const void* __restrict__ lab, int lab_dtype, int D, int H, int W,
                                             float x, float y, float z) {
    x = fminf(fmaxf(x, -2.0f), (float)W + 1.0f);
    y = fminf(fmaxf(y, -2.0f), (float)H + 1.0f);
    z = fminf(fmaxf(z, -2.0f), (float)D + 1.0f);
    const int rx = (int)rintf(x), ry = (int)rintf(y), rz = (int)rintf(z);
    if ((unsigned)rx < (unsigned)W && (unsigned)ry < (unsigned)H && (unsigned)rz < (unsigned)D)
        return ld_label(lab, lab_dtype, (rz * H + ry) * W + rx);
    return 0;
}

// Cell of a fixed-point position: the integer parts clamped into [-2, dim]
// (a cell there has every corner outside the volume, so the clamp changes no
// value or gradient, and it keeps quad indices inside the padded extent) and
// the fractions of the unclamped position.
__device__ __forceinline__ void fix_cell(const FixPos& P, int D, int H, int W, Cell& c) {
    c.ix = min(max(fix_floor(P.x), -2), W);
    c.iy = min(max(fix_floor(P.y), -2), H);
    c.iz = min(max(fix_floor(P.z), -2), D);
    c.fx = fix_frac(P.x);
    c.fy = fix_frac(P.y);
    c.fz = fix_frac(P.z);
}

template <typename VT>
__device__ __forceinline__ void load_cell_fix(const VT* __restrict__ vol, int D, int H, int W, const FixPos& P,
                                              Cell& c) {
    fix_cell(P, D, H, W, c);
    const int ix = c.ix, iy = c.iy, iz = c.iz;
    const int HW = H * W;
    const int base = (iz * H + iy) * W + ix;
    if ((unsigned)ix < (unsigned)(W - 1) && (unsigned)iy < (unsigned)(H - 1) && (unsigned)iz < (unsigned)(D - 1)) {
        c.v000 = ld_vox(vol, base);
        c.v001 = ld_vox(vol, base + 1);
        c.v010 = ld_vox(vol, base + W);
        c.v011 = ld_vox(vol, base + W + 1);
        c.v100 = ld_vox(vol, base + HW);
        c.v101 = ld_vox(vol, base + HW + 1);
        c.v110 = ld_vox(vol, base + HW + W);
        c.v111 = ld_vox(vol, base + HW + W + 1);
    } else {
        const bool x0 = (unsigned)ix < (unsigned)W, x1 = (unsigned)(ix + 1) < (unsigned)W;
        const bool y0 = (unsigned)iy < (unsigned)H, y1 = (unsigned)(iy + 1) < (unsigned)H;
        const bool z0 = (unsigned)iz < (unsigned)D, z1 = (unsigned)(iz + 1) < (unsigned)D;
        c.v000 = (z0 && y0 && x0) ? ld_vox(vol, base) : 0.f;
        c.v001 = (z0 && y0 && x1) ? ld_vox(vol, base + 1) : 0.f;
        c.v010 = (z0 && y1 && x0) ? ld_vox(vol, base + W) : 0.f;
        c.v011 = (z0 && y1 && x1) ? ld_vox(vol, base + W + 1) : 0.f;
        c.v100 = (z1 && y0 && x0) ? ld_vox(vol, base + HW) : 0.f;
        c.v101 = (z1 && y0 && x1) ? ld_vox(vol, base + HW + 1) : 0.f;
        c.v110 = (z1 && y1 && x0) ? ld_vox(vol, base + HW + W) : 0.f;
        c.v111 = (z1 && y1 && x1) ? ld_vox(vol, base + HW + W + 1) : 0.f;
    }
}

__device__ __forceinline__ int quad_index(const QuadGeom& g, const Cell& c) {
    return ((c.iz + 2) * g.qy + (c.iy + 2)) * g.qx + (c.ix + 2);
}

template <typename VT>
__device__ __forceinline__ void load_cell_quad_fix(const void* __restrict__ quad, const QuadGeom& g, int D, int H,
                                                   int W, const FixPos& P, Cell& c) {
    fix_cell(P, D, H, W, c);
    const int qi = quad_index(g, c);
    using Q = typename QuadOf<VT>::T;
    const Q* __restrict__ qp = reinterpret_cast<const Q*>(quad);
    const Q q0 = __ldg(qp + qi);
    const Q q1 = __ldg(qp + qi + g.plane);
    if constexpr (std::is_same<VT, float>::value) {
        unpack_quad(q0, c.v000, c.v001, c.v010, c.v011);
        unpack_quad(q1, c.v100, c.v101, c.v110, c.v111);
    } else if constexpr (std::is_same<VT, __nv_bfloat16>::value) {
        unpack_quad_bf16(q0, c.v000, c.v001, c.v010, c.v011);
        unpack_quad_bf16(q1, c.v100, c.v101, c.v110, c.v111);
    } else {
        unpack_quad_f16(q0, c.v000, c.v001, c.v010, c.v011);
        unpack_quad_f16(q1, c.v100, c.v101, c.v110, c.v111);
    }
}

// Labelled quad layout (16-bit volumes): a 16-byte element holds the four
// corner values of the plain 16-bit quad in .x/.y and the four corners'
// classes (uint8, in the same corner order; 255 = dropped, 0 outside the
// volume) in .z; .w is zero. The two loads of a sample then also carry the
// classes of its eight corners, and the nearest one is picked by rounding the
// exact position (ties to even, the reference's nearest rule): its offsets
// from the cell are 0 or 1 on each axis for any position the clamp left
// alone; any other offset means the nearest voxel is outside the volume,
// class 0.
template <typename VT>
__device__ __forceinline__ void load_cell_quad_labeled_fix(const void* __restrict__ quad, const QuadGeom& g, int D,
                                                           int H, int W, const FixPos& P, Cell& c) {
    fix_cell(P, D, H, W, c);
    const int qi = quad_index(g, c);
    const uint4* __restrict__ qp = reinterpret_cast<const uint4*>(quad);
    const uint4 q0 = __ldg(qp + qi);
    const uint4 q1 = __ldg(qp + qi + g.plane);
    if constexpr (std::is_same<VT, __nv_bfloat16>::value) {
        unpack_quad_bf16(make_uint2(q0.x, q0.y), c.v000, c.v001, c.v010, c.v011);
        unpack_quad_bf16(make_uint2(q1.x, q1.y), c.v100, c.v101, c.v110, c.v111);
    } else {
        unpack_quad_f16(make_uint2(q0.x, q0.y), c.v000, c.v001, c.v010, c.v011);
        unpack_quad_f16(make_uint2(q1.x, q1.y), c.v100, c.v101, c.v110, c.v111);
    }
    const int ox = fix_round(P.x) - c.ix, oy = fix_round(P.y) - c.iy, oz = fix_round(P.z) - c.iz;
    const bool inside = (unsigned)ox <= 1u && (unsigned)oy <= 1u && (unsigned)oz <= 1u;
    const unsigned labels = oz ? q1.z : q0.z;
    c.cls = inside ? (int)((labels >> (8 * (ox + 2 * oy))) & 0xffu) : 0;
}

// Nearest-voxel label at a fixed-point position (ties to even); positions
// whose nearest voxel is outside the volume read label 0 (zero padding).
__device__ __forceinline__ int nearest_label_fix(const void* __restrict__ lab, int lab_dtype, int D, int H, int W,
                                                 const FixPos& P) {
    const int rx = fix_round(P.x), ry = fix_round(P.y), rz = fix_round(P.z);
    if ((unsigned)rx < (unsigned)W && (unsigned)ry < (unsigned)H && (unsigned)rz < (unsigned)D)
        return ld_label(lab, lab_dtype, (rz * H + ry) * W + rx);
    return 0;
}

// --------------------------------------------------------------- tile layout
// A CTA owns a tile_w x tile_h patch of detector pixels; each warp owns an
// 8 x 4 sub-patch so that the 32 lanes of a gather hit a compact footprint
// in the plane across the rays.
struct TileMap {
    int IW, IH;      // image (or virtual image) extent in rays
    int tiles_x;     // tiles per image row
    int tiles;       // tiles per pose
    bool linear;     // rays are a flat list (virtual width 16)
};

__host__ __device__ __forceinline__ TileMap make_tilemap(int N, int width, int tw, int th) {
    TileMap m;
    m.linear = !(width > 0 && N % width == 0);
    m.IW = m.linear ? 16 : width;
    m.IH = m.linear ? (N + 15) / 16 : N / width;
    m.tiles_x = (m.IW + tw - 1) / tw;
    m.tiles = m.tiles_x * ((m.IH + th - 1) / th);
    return m;
}

// Ray index of lane `r` (0 <= r < tw * th) of tile `tile`, or -1 if padding.
// tw is a multiple of 8 and th a multiple of 4.
__device__ __forceinline__ int tile_ray(const TileMap& m, int N, int tw, int th, int tile, int r) {
    const int warp = r >> 5, lane = r & 31;
    const int wpr = tw >> 3;  // warps per tile row
    const int tx = tile % m.tiles_x, ty = tile / m.tiles_x;
    const int px = tx * tw + (warp % wpr) * 8 + (lane & 7);
    const int py = ty * th + (warp / wpr) * 4 + (lane >> 3);
    if (px >= m.IW || py >= m.IH) return -1;
    const int n = py * m.IW + px;
    return n < N ? n : -1;
}

}  // namespace ndrr
