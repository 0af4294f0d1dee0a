// Ray-march forward and adjoint kernels for sm_103a, plus their launchers.
//
// Work decomposition: one CTA per (pose, detector tile). A tile is
// tile_w x tile_h rays, each warp an 8 x 4 sub-patch so that its gathers hit a
// compact footprint. Optionally each ray's sample window is split into
// `sample_split` contiguous chunks marched by different threads of the same
// CTA; the chunk partials are summed in shared memory in a fixed order, so the
// result is deterministic and no global partial buffer or second pass is
// needed for the forward (the reference writes split partials to global
// memory and sums them in torch, nanodrr src/nanodrr/drr/_fused.py:436-459).
//
// Forward per sample (reference _fused.py:190-228, 300): trilinear tap with
// zero padding, optional nearest-label routing, fp32 accumulation; the sum is
// scaled by the per-ray step at the end (_fused.py:327-331).
//
// Adjoint per sample (reference _fused.py:230-298): recompute the tap, form
// g = go[b, class, n] * step, the analytic trilinear position gradient, the
// pose partial dL/dM_ij += g * dv_i * [q, 1]_j, optional camera-space
// gradients, and the volume gradient scattered to the 8 corners by atomics.
// Pose partials are reduced per CTA with a fixed shuffle tree and per pose by
// a second small kernel in a fixed order, so gM is bitwise reproducible.
#include <algorithm>
#include <cstdio>
#include <string>

#include "ndrr_device.cuh"
#include "ndrr_launch.h"

namespace ndrr {

struct MarchParams {
    const void* vol;
    int D, H, W;
    const void* lab;
    int lab_dtype;
    int C;
    const float* M;
    const float* src;
    const float* tgt;
    const float* step;
    int src_per_ray;
    int B, N, S;
    float inv_s;
    const float* t_window;
    // forward
    void* out;
    void* out_total;
    // adjoint
    const void* go;
    int go_dtype;
    float* gvol;
    float* gsrc;
    float* gtgt;
    float* gstep;
    float* partials;  // [B * tiles, kPartialStride]
    // launch shape
    TileMap tm;
    int tw, th, K;
};

constexpr int kPartialStride = 16;  // 12 pose terms + 3 shared-source terms + pad

// Per-thread ray set-up: voxel-space line, window, this thread's chunk.
struct ThreadRay {
    Ray ray;
    int n;         // ray index or -1
    size_t bn;     // b * N + n
    float stepv;   // camera-space sample spacing
    float sx, sy, sz, ex, ey, ez;  // camera-space source and src -> tgt
    int s0, s1;    // this thread's sample chunk
};

__device__ __forceinline__ void setup_thread_ray(const MarchParams& p, const float (&m)[12], int b, int n, int k,
                                                 ThreadRay& tr) {
    tr.n = n;
    tr.ray.lo = tr.ray.hi = 0;
    tr.stepv = 0.f;
    tr.sx = tr.sy = tr.sz = tr.ex = tr.ey = tr.ez = 0.f;
    tr.ray.p0x = tr.ray.p0y = tr.ray.p0z = tr.ray.dx = tr.ray.dy = tr.ray.dz = 0.f;
    tr.bn = 0;
    if (n >= 0) {
        const size_t bn = (size_t)b * p.N + n;
        tr.bn = bn;
        const float* sp = p.src_per_ray ? p.src + bn * 3 : p.src + (size_t)b * 3;
        const float sx = __ldg(sp + 0), sy = __ldg(sp + 1), sz = __ldg(sp + 2);
        const float tx = __ldg(p.tgt + bn * 3 + 0), ty = __ldg(p.tgt + bn * 3 + 1), tz = __ldg(p.tgt + bn * 3 + 2);
        const float ex = tx - sx, ey = ty - sy, ez = tz - sz;
        tr.sx = sx; tr.sy = sy; tr.sz = sz;
        tr.ex = ex; tr.ey = ey; tr.ez = ez;
        tr.ray.p0x = m[0] * sx + m[1] * sy + m[2] * sz + m[3];
        tr.ray.p0y = m[4] * sx + m[5] * sy + m[6] * sz + m[7];
        tr.ray.p0z = m[8] * sx + m[9] * sy + m[10] * sz + m[11];
        tr.ray.dx = m[0] * ex + m[1] * ey + m[2] * ez;
        tr.ray.dy = m[4] * ex + m[5] * ey + m[6] * ez;
        tr.ray.dz = m[8] * ex + m[9] * ey + m[10] * ez;
        ray_window(tr.ray, p.D, p.H, p.W, p.S);
        if (p.t_window) apply_t_window(tr.ray, __ldg(p.t_window + bn * 2), __ldg(p.t_window + bn * 2 + 1), p.S);
        tr.stepv = __ldg(p.step + bn);
    }
    const int len = max(tr.ray.hi - tr.ray.lo, 0);
    const int chunk = (len + p.K - 1) / p.K;
    tr.s0 = tr.ray.lo + k * chunk;
    tr.s1 = min(tr.ray.hi, tr.s0 + chunk);
}

// ===================================================================== forward
template <typename VT, typename OT, bool MULTI>
__global__ void __launch_bounds__(512, 2) raymarch_fwd_kernel(const MarchParams p) {
    extern __shared__ float smem[];
    const int R = p.tw * p.th;
    const int NT = R * p.K;
    const int tid = threadIdx.x;
    const int r = tid % R, k = tid / R;
    const int tile = blockIdx.x % p.tm.tiles;
    const int b = blockIdx.x / p.tm.tiles;
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, r);

    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);

    ThreadRay tr;
    setup_thread_ray(p, m, b, n, k, tr);

    const VT* __restrict__ vol = reinterpret_cast<const VT*>(p.vol);
    float acc = 0.f;
    float* cacc = smem + tid;  // MULTI: per-thread class accumulators, stride NT
    if (MULTI) {
        for (int c = 0; c < p.C; ++c) cacc[c * NT] = 0.f;
    }
    for (int s = tr.s0; s < tr.s1; ++s) {
        const float t = (float)s * p.inv_s;
        const float x = fmaf(t, tr.ray.dx, tr.ray.p0x);
        const float y = fmaf(t, tr.ray.dy, tr.ray.p0y);
        const float z = fmaf(t, tr.ray.dz, tr.ray.p0z);
        Cell cell;
        load_cell(vol, p.D, p.H, p.W, x, y, z, cell);
        const float val = cell_value(cell);
        acc += val;
        if (MULTI) {
            const int cls = nearest_label(p.lab, p.lab_dtype, p.D, p.H, p.W, x, y, z);
            if ((unsigned)cls < (unsigned)p.C) cacc[cls * NT] += val;
        }
    }

    // Sum the K chunk partials of each ray in a fixed order.
    float* red = smem + (MULTI ? (size_t)p.C * NT : 0);
    red[tid] = acc;
    __syncthreads();
    OT* out = reinterpret_cast<OT*>(p.out);
    OT* out_total = reinterpret_cast<OT*>(p.out_total);
    if (!MULTI) {
        if (k == 0 && n >= 0) {
            float sum = red[r];
            for (int j = 1; j < p.K; ++j) sum += red[r + j * R];
            st_out(out, tr.bn, sum * tr.stepv);
            if (out_total) st_out(out_total, tr.bn, sum * tr.stepv);
        }
    } else {
        if (out_total && k == 0 && n >= 0) {
            float sum = red[r];
            for (int j = 1; j < p.K; ++j) sum += red[r + j * R];
            st_out(out_total, tr.bn, sum * tr.stepv);
        }
        // Channel write-out: consecutive threads take consecutive rays of one
        // channel, so stores coalesce along the detector rows.
        for (int idx = tid; idx < R * p.C; idx += NT) {
            const int rr = idx % R, c = idx / R;
            const int nn = tile_ray(p.tm, p.N, p.tw, p.th, tile, rr);
            if (nn < 0) continue;
            float sum = smem[(size_t)c * NT + rr];
            for (int j = 1; j < p.K; ++j) sum += smem[(size_t)c * NT + rr + j * R];
            const size_t bn = (size_t)b * p.N + nn;
            st_out(out, ((size_t)b * p.C + c) * p.N + nn, sum * __ldg(p.step + bn));
        }
    }
}

// ===================================================================== adjoint
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename VT, bool MULTI, bool GVOL, bool GCAM>
__global__ void __launch_bounds__(512, 1) raymarch_bwd_kernel(const MarchParams p) {
    extern __shared__ float smem[];
    const int R = p.tw * p.th;
    const int NT = R * p.K;
    const int tid = threadIdx.x;
    const int r = tid % R, k = tid / R;
    const int tile = blockIdx.x % p.tm.tiles;
    const int b = blockIdx.x / p.tm.tiles;
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, r);

    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);

    ThreadRay tr;
    setup_thread_ray(p, m, b, n, k, tr);

    const VT* __restrict__ vol = reinterpret_cast<const VT*>(p.vol);
    const int HW = p.H * p.W;

    float a[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) a[j] = 0.f;
    float gsx = 0.f, gsy = 0.f, gsz = 0.f, gtx = 0.f, gty = 0.f, gtz = 0.f, gst = 0.f;

    float go_ray = 0.f;
    if (!MULTI && n >= 0) go_ray = ld_any_f(p.go, p.go_dtype, tr.bn);

    for (int s = tr.s0; s < tr.s1; ++s) {
        const float t = (float)s * p.inv_s;
        const float x = fmaf(t, tr.ray.dx, tr.ray.p0x);
        const float y = fmaf(t, tr.ray.dy, tr.ray.p0y);
        const float z = fmaf(t, tr.ray.dz, tr.ray.p0z);
        float gg = go_ray;
        if (MULTI) {
            // Upstream gradient of this sample's channel; out-of-range labels
            // are masked like the forward drops them (_fused.py:233-237).
            const int cls = nearest_label(p.lab, p.lab_dtype, p.D, p.H, p.W, x, y, z);
            gg = ((unsigned)cls < (unsigned)p.C)
                     ? ld_any_f(p.go, p.go_dtype, ((size_t)b * p.C + cls) * p.N + tr.n)
                     : 0.f;
        }
        // Every adjoint term of this sample is proportional to gg.
        if (gg == 0.f) continue;
        const float g = gg * tr.stepv;
        Cell cell;
        load_cell(vol, p.D, p.H, p.W, x, y, z, cell);
        float dvx, dvy, dvz;
        cell_grad(cell, dvx, dvy, dvz);
        const float gx = g * dvx, gy = g * dvy, gz = g * dvz;
        const float qx = fmaf(t, tr.ex, tr.sx), qy = fmaf(t, tr.ey, tr.sy), qz = fmaf(t, tr.ez, tr.sz);
        a[0] = fmaf(gx, qx, a[0]);
        a[1] = fmaf(gx, qy, a[1]);
        a[2] = fmaf(gx, qz, a[2]);
        a[3] += gx;
        a[4] = fmaf(gy, qx, a[4]);
        a[5] = fmaf(gy, qy, a[5]);
        a[6] = fmaf(gy, qz, a[6]);
        a[7] += gy;
        a[8] = fmaf(gz, qx, a[8]);
        a[9] = fmaf(gz, qy, a[9]);
        a[10] = fmaf(gz, qz, a[10]);
        a[11] += gz;
        if (GCAM) {
            // Chain to camera space: gq = M[:, :3]^T gpos.
            const float gqx = m[0] * gx + m[4] * gy + m[8] * gz;
            const float gqy = m[1] * gx + m[5] * gy + m[9] * gz;
            const float gqz = m[2] * gx + m[6] * gy + m[10] * gz;
            const float omt = 1.f - t;
            gsx = fmaf(omt, gqx, gsx);
            gsy = fmaf(omt, gqy, gsy);
            gsz = fmaf(omt, gqz, gsz);
            gtx = fmaf(t, gqx, gtx);
            gty = fmaf(t, gqy, gty);
            gtz = fmaf(t, gqz, gtz);
            gst = fmaf(gg, cell_value(cell), gst);
        }
        if (GVOL) {
            const float wx1 = cell.fx, wy1 = cell.fy, wz1 = cell.fz;
            const float wx0 = 1.f - wx1, wy0 = 1.f - wy1, wz0 = 1.f - wz1;
            const int ix = cell.ix, iy = cell.iy, iz = cell.iz;
            const int base = (iz * p.H + iy) * p.W + ix;
            const float g00 = g * wz0 * wy0, g01 = g * wz0 * wy1, g10 = g * wz1 * wy0, g11 = g * wz1 * wy1;
            if ((unsigned)ix < (unsigned)(p.W - 1) && (unsigned)iy < (unsigned)(p.H - 1) &&
                (unsigned)iz < (unsigned)(p.D - 1)) {
                atomicAdd(p.gvol + base, g00 * wx0);
                atomicAdd(p.gvol + base + 1, g00 * wx1);
                atomicAdd(p.gvol + base + p.W, g01 * wx0);
                atomicAdd(p.gvol + base + p.W + 1, g01 * wx1);
                atomicAdd(p.gvol + base + HW, g10 * wx0);
                atomicAdd(p.gvol + base + HW + 1, g10 * wx1);
                atomicAdd(p.gvol + base + HW + p.W, g11 * wx0);
                atomicAdd(p.gvol + base + HW + p.W + 1, g11 * wx1);
            } else {
                const bool x0 = (unsigned)ix < (unsigned)p.W, x1 = (unsigned)(ix + 1) < (unsigned)p.W;
                const bool y0 = (unsigned)iy < (unsigned)p.H, y1 = (unsigned)(iy + 1) < (unsigned)p.H;
                const bool z0 = (unsigned)iz < (unsigned)p.D, z1 = (unsigned)(iz + 1) < (unsigned)p.D;
                if (z0 && y0 && x0) atomicAdd(p.gvol + base, g00 * wx0);
                if (z0 && y0 && x1) atomicAdd(p.gvol + base + 1, g00 * wx1);
                if (z0 && y1 && x0) atomicAdd(p.gvol + base + p.W, g01 * wx0);
                if (z0 && y1 && x1) atomicAdd(p.gvol + base + p.W + 1, g01 * wx1);
                if (z1 && y0 && x0) atomicAdd(p.gvol + base + HW, g10 * wx0);
                if (z1 && y0 && x1) atomicAdd(p.gvol + base + HW + 1, g10 * wx1);
                if (z1 && y1 && x0) atomicAdd(p.gvol + base + HW + p.W, g11 * wx0);
                if (z1 && y1 && x1) atomicAdd(p.gvol + base + HW + p.W + 1, g11 * wx1);
            }
        }
    }

    // ---- CTA reduction of the pose partials (fixed order: deterministic).
    const bool shared_src = GCAM && !p.src_per_ray;
    const int nwarps = NT >> 5;
    const int warp = tid >> 5, lane = tid & 31;
    float* wred = smem;  // [nwarps][kPartialStride]
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        const float v = warp_sum(a[j]);
        if (lane == 0) wred[warp * kPartialStride + j] = v;
    }
    if (shared_src) {
        const float v0 = warp_sum(gsx), v1 = warp_sum(gsy), v2 = warp_sum(gsz);
        if (lane == 0) {
            wred[warp * kPartialStride + 12] = v0;
            wred[warp * kPartialStride + 13] = v1;
            wred[warp * kPartialStride + 14] = v2;
        }
    }
    __syncthreads();
    const int nterms = shared_src ? 15 : 12;
    if (tid < nterms) {
        float sum = wred[tid];
        for (int w = 1; w < nwarps; ++w) sum += wred[w * kPartialStride + tid];
        p.partials[(size_t)blockIdx.x * kPartialStride + tid] = sum;
    }

    // ---- Per-ray camera gradients: sum the K chunk partials in order.
    if (GCAM) {
        __syncthreads();
        float* cr = smem;  // [7][NT]
        cr[0 * NT + tid] = gtx;
        cr[1 * NT + tid] = gty;
        cr[2 * NT + tid] = gtz;
        cr[3 * NT + tid] = gst;
        cr[4 * NT + tid] = gsx;
        cr[5 * NT + tid] = gsy;
        cr[6 * NT + tid] = gsz;
        __syncthreads();
        if (k == 0 && n >= 0) {
            float v[7];
#pragma unroll
            for (int q = 0; q < 7; ++q) {
                float sum = cr[q * NT + r];
                for (int j = 1; j < p.K; ++j) sum += cr[q * NT + r + j * R];
                v[q] = sum;
            }
            p.gtgt[tr.bn * 3 + 0] = v[0];
            p.gtgt[tr.bn * 3 + 1] = v[1];
            p.gtgt[tr.bn * 3 + 2] = v[2];
            p.gstep[tr.bn] = v[3];
            if (p.src_per_ray) {
                p.gsrc[tr.bn * 3 + 0] = v[4];
                p.gsrc[tr.bn * 3 + 1] = v[5];
                p.gsrc[tr.bn * 3 + 2] = v[6];
            }
        }
    }
}

// Per-pose sum of the per-tile partials in a fixed order. One CTA per pose.
__global__ void __launch_bounds__(256) pose_partials_reduce_kernel(const float* __restrict__ partials, int tiles,
                                                                   float* __restrict__ gM,
                                                                   float* __restrict__ gsrc_shared) {
    __shared__ float red[8][16];
    const int b = blockIdx.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nterms = gsrc_shared ? 15 : 12;
    for (int j = 0; j < nterms; ++j) {
        float v = 0.f;
        for (int t = tid; t < tiles; t += blockDim.x) v += partials[((size_t)b * tiles + t) * kPartialStride + j];
        v = warp_sum(v);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (tid < nterms) {
        float sum = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += red[w][tid];
        if (tid < 12)
            gM[(size_t)b * 12 + tid] = sum;
        else
            gsrc_shared[(size_t)b * 3 + (tid - 12)] = sum;
    }
}

// ==================================================================== launchers
static MarchParams make_params(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    MarchParams p{};
    p.vol = a.vol;
    p.D = a.D;
    p.H = a.H;
    p.W = a.W;
    p.lab = a.lab;
    p.lab_dtype = a.lab_dtype;
    p.C = a.n_classes;
    p.M = a.M;
    p.src = a.src;
    p.tgt = a.tgt;
    p.step = a.step;
    p.src_per_ray = a.src_per_ray;
    p.B = a.B;
    p.N = a.N;
    p.S = a.n_samples;
    p.inv_s = 1.0f / (float)(a.n_samples - 1);
    p.t_window = a.t_window;
    p.out = a.out;
    p.out_total = a.out_total;
    p.go = a.go;
    p.go_dtype = a.go_dtype;
    p.gvol = a.gvol;
    p.gsrc = a.gsrc;
    p.gtgt = a.gtgt;
    p.gstep = a.gstep;
    p.partials = reinterpret_cast<float*>(a.workspace);
    p.tw = ls.tw;
    p.th = ls.th;
    p.K = ls.K;
    p.tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
    return p;
}

LaunchShape choose_shape(const ndrr_raymarch_args& a, int sm_count) {
    LaunchShape ls;
    ls.tw = a.tile_w > 0 ? a.tile_w : 16;
    ls.th = a.tile_h > 0 ? a.tile_h : 8;
    if (a.sample_split > 0) {
        ls.K = a.sample_split;
    } else {
        // Split each ray's samples across threads only when the rays alone
        // leave the GPU under-filled (about 1024 resident threads per SM).
        const TileMap tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
        const double threads = (double)a.B * tm.tiles * ls.tw * ls.th;
        const double want = (double)sm_count * 1024.0;
        ls.K = threads >= want ? 1 : (threads * 2 >= want ? 2 : 4);
        if (ls.tw * ls.th * ls.K > 512) ls.K = std::max(1, 512 / (ls.tw * ls.th));
    }
    return ls;
}

uint64_t bwd_workspace_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    const TileMap tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
    return (uint64_t)a.B * tm.tiles * kPartialStride * sizeof(float);
}

size_t fwd_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    const size_t NT = (size_t)ls.tw * ls.th * ls.K;
    return (a.n_classes > 1 ? (size_t)a.n_classes + 1 : 1) * NT * sizeof(float);
}

size_t bwd_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    const size_t NT = (size_t)ls.tw * ls.th * ls.K;
    const size_t wred = (NT / 32) * kPartialStride;
    const size_t cam = a.need_gcam ? 7 * NT : 0;
    return std::max(wred, cam) * sizeof(float);
}

template <typename Kern>
static cudaError_t launch_kernel(Kern kern, unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                                 const MarchParams& p) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, block, smem, st>>>(p);
    return cudaGetLastError();
}

template <typename VT, typename OT>
static cudaError_t fwd_dispatch_multi(const MarchParams& p, bool multi, unsigned grid, unsigned block, size_t smem,
                                      cudaStream_t st) {
    if (multi) return launch_kernel(raymarch_fwd_kernel<VT, OT, true>, grid, block, smem, st, p);
    return launch_kernel(raymarch_fwd_kernel<VT, OT, false>, grid, block, smem, st, p);
}

template <typename VT>
static cudaError_t fwd_dispatch_out(const MarchParams& p, int out_dtype, bool multi, unsigned grid, unsigned block,
                                    size_t smem, cudaStream_t st) {
    switch (out_dtype) {
        case NDRR_F32: return fwd_dispatch_multi<VT, float>(p, multi, grid, block, smem, st);
        case NDRR_F16: return fwd_dispatch_multi<VT, __half>(p, multi, grid, block, smem, st);
        case NDRR_BF16: return fwd_dispatch_multi<VT, __nv_bfloat16>(p, multi, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fwd(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st) {
    const MarchParams p = make_params(a, ls);
    const unsigned grid = (unsigned)((size_t)a.B * p.tm.tiles);
    const unsigned block = (unsigned)(ls.tw * ls.th * ls.K);
    const size_t smem = fwd_smem_bytes(a, ls);
    const bool multi = a.n_classes > 1;
    switch (a.vol_dtype) {
        case NDRR_F32: return fwd_dispatch_out<float>(p, a.out_dtype, multi, grid, block, smem, st);
        case NDRR_F16: return fwd_dispatch_out<__half>(p, a.out_dtype, multi, grid, block, smem, st);
        case NDRR_BF16: return fwd_dispatch_out<__nv_bfloat16>(p, a.out_dtype, multi, grid, block, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

template <typename VT, bool MULTI>
static cudaError_t bwd_dispatch_flags(const MarchParams& p, bool gvol, bool gcam, unsigned grid, unsigned block,
                                      size_t smem, cudaStream_t st) {
    if (gvol && gcam) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, true>, grid, block, smem, st, p);
    if (gvol) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, true, false>, grid, block, smem, st, p);
    if (gcam) return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, true>, grid, block, smem, st, p);
    return launch_kernel(raymarch_bwd_kernel<VT, MULTI, false, false>, grid, block, smem, st, p);
}

template <typename VT>
static cudaError_t bwd_dispatch(const MarchParams& p, bool multi, bool gvol, bool gcam, unsigned grid,
                                unsigned block, size_t smem, cudaStream_t st) {
    if (multi) return bwd_dispatch_flags<VT, true>(p, gvol, gcam, grid, block, smem, st);
    return bwd_dispatch_flags<VT, false>(p, gvol, gcam, grid, block, smem, st);
}

cudaError_t launch_bwd(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st) {
    const MarchParams p = make_params(a, ls);
    const unsigned grid = (unsigned)((size_t)a.B * p.tm.tiles);
    const unsigned block = (unsigned)(ls.tw * ls.th * ls.K);
    const size_t smem = bwd_smem_bytes(a, ls);
    const bool multi = a.n_classes > 1, gvol = a.need_gvol != 0, gcam = a.need_gcam != 0;
    cudaError_t e;
    switch (a.vol_dtype) {
        case NDRR_F32: e = bwd_dispatch<float>(p, multi, gvol, gcam, grid, block, smem, st); break;
        case NDRR_F16: e = bwd_dispatch<__half>(p, multi, gvol, gcam, grid, block, smem, st); break;
        case NDRR_BF16: e = bwd_dispatch<__nv_bfloat16>(p, multi, gvol, gcam, grid, block, smem, st); break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    float* gsrc_shared = (a.need_gcam && !a.src_per_ray) ? a.gsrc : nullptr;
    pose_partials_reduce_kernel<<<a.B, 256, 0, st>>>(p.partials, p.tm.tiles, a.gM, gsrc_shared);
    return cudaGetLastError();
}

}  // namespace ndrr
