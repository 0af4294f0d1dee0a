// Shared device code of the ray-march kernels: parameters, per-ray set-up,
// empty-space skipping, the forward body and the adjoint bodies. The kernels
// are templates instantiated by the launchers in ndrr_fwd.cu, ndrr_bwd.cu and
// ndrr_brick.cu (separate translation units, compiled in parallel).
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
#pragma once

#include <algorithm>
#include <climits>
#include <cstdio>

#include "ndrr_device.cuh"
#include "ndrr_launch.h"
#include "ndrr_proposal.cuh"
#include "ndrr_skip.cuh"

namespace ndrr {

struct MarchParams {
    const void* vol;
    int D, H, W;
    const void* lab;
    int lab_dtype;
    int C;
    const float* M;
    const float* M_lo;  // optional low parts: M + M_lo is the affine to ~2^-48 (NULL: M is exact)
    const float* src;
    const float* tgt;
    const float* step;
    int src_per_ray;
    int B, N, S;
    float inv_s;
    const float* t_window;
    const int* win;  // per-ray sample windows [B * N][2] or NULL
    const int* gwin;  // volume-gradient adjoint: gather windows [B * N][2] (samples outside
                      // them have eight zero corners: scattered without loading) or NULL
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
    // empty-space skipping
    int skip_mode;
    OccGrid occ;
    const unsigned char* proposal;  // packed network parameters
    float margin;                   // widening of a proposed interval (samples)
    unsigned long long* stats;      // [4] counters or NULL
    float* out_extent;              // [B, N, 2] or NULL
    // quad layout (gathers from `quad`, volume-gradient scatter into `gquad`)
    const void* quad;
    float* gquad;
    QuadGeom qg;
    // launch shape
    TileMap tm;
    int tw, th, K;
};

constexpr int kSkipSteps = 256;  // distance-field steps per query before giving up

constexpr int kPartialStride = 16;  // 12 pose terms + 3 shared-source terms + pad

// Per-thread ray set-up: voxel-space line, window, this thread's chunk.
struct ThreadRay {
    Ray ray;
    int n;         // ray index or -1
    size_t bn;     // b * N + n
    float stepv;   // camera-space sample spacing
    float sx, sy, sz, ex, ey, ez;  // camera-space source and src -> tgt
    int s0, s1;    // this thread's sample chunk
    FixPos f0, fd;  // voxel-space position of sample 0 and the step per sample, 32.32 fixed point
    int glo, ghi;   // samples whose corners are loaded (all outside have zero corners)
};

// Fixed-point start and step of a ray: p0 = M [src, 1] and step = M [tgt -
// src, 0] / (S - 1) in float-float from the float32 inputs (tgt - src exactly,
// M as M + M_lo), converted to 32.32 fixed point.
__device__ __forceinline__ void fix_ray(const MarchParams& p, const float (&m)[12], int b, float sx, float sy,
                                        float sz, float tx, float ty, float tz, ThreadRay& tr) {
    const F2 e[3] = {f2_two_sum(tx, -sx), f2_two_sum(ty, -sy), f2_two_sum(tz, -sz)};
    const F2 src[3] = {F2{sx, 0.f}, F2{sy, 0.f}, F2{sz, 0.f}};
    const float n1 = (float)(p.S - 1);
    long long f0[3], fd[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        F2 row[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) row[j] = F2{m[4 * i + j], p.M_lo ? __ldg(p.M_lo + (size_t)b * 12 + 4 * i + j) : 0.f};
        const F2 d = f2_add(f2_add(f2_mul(row[0], e[0]), f2_mul(row[1], e[1])), f2_mul(row[2], e[2]));
        const F2 q = f2_add(f2_add(f2_add(f2_mul(row[0], src[0]), f2_mul(row[1], src[1])), f2_mul(row[2], src[2])),
                            row[3]);
        f0[i] = f2_to_fix(q);
        fd[i] = f2_to_fix(f2_div_int(d, n1));
    }
    tr.f0 = FixPos{f0[0], f0[1], f0[2]};
    tr.fd = FixPos{fd[0], fd[1], fd[2]};
}

// Fixed-point position of sample s.
__device__ __forceinline__ FixPos fix_at(const ThreadRay& tr, int s) {
    return FixPos{tr.f0.x + (long long)s * tr.fd.x, tr.f0.y + (long long)s * tr.fd.y, tr.f0.z + (long long)s * tr.fd.z};
}

// Box-culled ray set-up (every thread of a ray computes the same window).
__device__ __forceinline__ void init_thread_ray(const MarchParams& p, const float (&m)[12], int b, int n,
                                                ThreadRay& tr) {
    tr.n = n;
    tr.ray.lo = tr.ray.hi = 0;
    tr.stepv = 0.f;
    tr.sx = tr.sy = tr.sz = tr.ex = tr.ey = tr.ez = 0.f;
    tr.ray.p0x = tr.ray.p0y = tr.ray.p0z = tr.ray.dx = tr.ray.dy = tr.ray.dz = 0.f;
    tr.f0 = tr.fd = FixPos{0, 0, 0};
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
        fix_ray(p, m, b, sx, sy, sz, tx, ty, tz, tr);
        ray_window(tr.ray, p.D, p.H, p.W, p.S);
        if (p.t_window) apply_t_window(tr.ray, __ldg(p.t_window + bn * 2), __ldg(p.t_window + bn * 2 + 1), p.S);
        if (p.win) {
            const int2 w = __ldg(reinterpret_cast<const int2*>(p.win) + bn);
            tr.ray.lo = max(tr.ray.lo, w.x);
            tr.ray.hi = max(min(tr.ray.hi, w.y), tr.ray.lo);
        }
        tr.stepv = __ldg(p.step + bn);
    }
    tr.s0 = tr.ray.lo;
    tr.s1 = tr.ray.hi;
    tr.glo = 0;
    tr.ghi = INT_MAX;
}

// This thread's share [s0, s1) of the ray's window when K threads split it.
__device__ __forceinline__ void chunk_thread_ray(ThreadRay& tr, int k, int K) {
    const int len = max(tr.ray.hi - tr.ray.lo, 0);
    const int chunk = (len + K - 1) / K;
    tr.s0 = tr.ray.lo + k * chunk;
    tr.s1 = min(tr.ray.hi, tr.s0 + chunk);
}

__device__ __forceinline__ void setup_thread_ray(const MarchParams& p, const float (&m)[12], int b, int n, int k,
                                                 ThreadRay& tr) {
    init_thread_ray(p, m, b, n, tr);
    chunk_thread_ray(tr, k, p.K);
}

// Narrow the box-culled window of a ray with the occupancy grid.
//  NDRR_SKIP_OCCUPANCY: march the distance field from both ends of the window
//  to the first occupied cell; every sample outside [t_near, t_far] lies in an
//  empty cell. NDRR_SKIP_PROPOSAL: keep the proposed [pn, pf] only if the
//  distance field shows both outer segments empty, else keep the full window
//  (a fallback). Returns true when the ray fell back.
__device__ __forceinline__ bool apply_skip(const MarchParams& p, ThreadRay& tr, float pn, float pf) {
    Ray& r = tr.ray;
    if (tr.n < 0 || r.lo >= r.hi) return false;
    const float sm1 = (float)(p.S - 1);
    const float tb0 = (float)r.lo * p.inv_s, tb1 = (float)(r.hi - 1) * p.inv_s;
    float tn, tf;
    if (p.skip_mode == NDRR_SKIP_OCCUPANCY) {
        const int h1 = first_occupied(p.occ, r, tb0, tb1, kSkipSteps, &tn);
        if (h1 == 0) {
            r.hi = r.lo;  // nothing occupied along the window
            return false;
        }
        if (h1 < 0) return true;
        const int h2 = first_occupied(p.occ, r, tb1, tn, kSkipSteps, &tf);
        if (h2 != 1) tf = tb1;
    } else {
        tn = pn - p.margin * p.inv_s;
        tf = pf + p.margin * p.inv_s;
        float unused;
        if (tn > tf) {
            // Proposed empty: the two outer segments cover the whole window,
            // so one walk over it decides.
            if (first_occupied(p.occ, r, tb0, tb1, kSkipSteps, &unused) != 0) return true;
            r.hi = r.lo;
            return false;
        }
        if (first_occupied(p.occ, r, tb0, fminf(tn, tb1), kSkipSteps, &unused) != 0) return true;
        if (first_occupied(p.occ, r, tb1, fmaxf(tf, tb0), kSkipSteps, &unused) != 0) return true;
    }
    // Keep one extra sample on each side of [tn, tf].
    const float a = fminf(fmaxf(floorf(tn * sm1) - 1.0f, (float)r.lo), (float)r.hi);
    const float e = fminf(fmaxf(ceilf(tf * sm1) + 2.0f, (float)r.lo), (float)r.hi);
    r.lo = (int)a;
    r.hi = max((int)e, r.lo);
    return false;
}

// Accumulate the CTA's skip counters into p.stats (one atomic per counter).
__device__ __forceinline__ void skip_stats_add(const MarchParams& p, unsigned long long* sstat, int k, bool has,
                                               bool fell, int box_len, int len) {
    if (k == 0) {
        unsigned v0 = __ballot_sync(0xffffffffu, has), v1 = __ballot_sync(0xffffffffu, fell);
        unsigned long long l = (unsigned long long)len, bl = (unsigned long long)box_len;
        for (int o = 16; o > 0; o >>= 1) {
            l += __shfl_xor_sync(0xffffffffu, l, o);
            bl += __shfl_xor_sync(0xffffffffu, bl, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(sstat + 0, (unsigned long long)__popc(v0));
            atomicAdd(sstat + 1, (unsigned long long)__popc(v1));
            atomicAdd(sstat + 2, l);
            atomicAdd(sstat + 3, bl);
        }
    }
}

// Volume layouts a kernel reads (the QUAD template argument).
constexpr int kLayoutVolume = 0;   // the caller's [D, H, W] array, eight gathers
constexpr int kLayoutQuad = 1;     // quad layout, two vector loads
constexpr int kLayoutQuadLab = 2;  // labelled quad layout (16-bit volumes): classes ride in the same loads

// The eight corners of the sample's cell from the plain volume (bounds
// checked per corner) or from the quad layouts (two vector loads), at a
// float position (the forward) or a fixed-point one (the adjoint).
template <typename VT, int QUAD>
__device__ __forceinline__ void fetch_cell(const MarchParams& p, float x, float y, float z, Cell& c) {
    if constexpr (QUAD == kLayoutQuadLab) {
        load_cell_quad_labeled<VT>(p.quad, p.qg, p.D, p.H, p.W, x, y, z, c);
    } else if constexpr (QUAD == kLayoutQuad) {
        load_cell_quad<VT>(p.quad, p.qg, p.D, p.H, p.W, x, y, z, c);
    } else {
        load_cell(reinterpret_cast<const VT*>(p.vol), p.D, p.H, p.W, x, y, z, c);
    }
}

// The cell of a sample known to have eight zero corners: its position and
// weights, no loads.
__device__ __forceinline__ void zero_cell(const MarchParams& p, const FixPos& P, Cell& c) {
    fix_cell(P, p.D, p.H, p.W, c);
    c.v000 = c.v001 = c.v010 = c.v011 = c.v100 = c.v101 = c.v110 = c.v111 = 0.f;
    c.cls = 0;
}

template <typename VT, int QUAD>
__device__ __forceinline__ void fetch_cell(const MarchParams& p, const FixPos& P, Cell& c) {
    if constexpr (QUAD == kLayoutQuadLab) {
        load_cell_quad_labeled_fix<VT>(p.quad, p.qg, p.D, p.H, p.W, P, c);
    } else if constexpr (QUAD == kLayoutQuad) {
        load_cell_quad_fix<VT>(p.quad, p.qg, p.D, p.H, p.W, P, c);
    } else {
        load_cell_fix(reinterpret_cast<const VT*>(p.vol), p.D, p.H, p.W, P, c);
    }
}

// ===================================================================== forward
// SKIP: 0 no skipping (or precomputed sample windows), 1 occupancy window.
template <typename VT, typename OT, bool MULTI, int SKIP, int QUAD = kLayoutVolume>
__device__ __forceinline__ void fwd_body(const MarchParams& p, const int tile, const int b) {
    extern __shared__ float smem[];
    const int R = p.tw * p.th;
    const int NT = R * p.K;
    const int tid = threadIdx.x;
    const int r = tid % R, k = tid / R;
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, r);

    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);

    ThreadRay tr;
    init_thread_ray(p, m, b, n, tr);
    if (SKIP != 0) {
        const int box_len = max(tr.ray.hi - tr.ray.lo, 0);
        const bool has = n >= 0 && box_len > 0;
        const bool fell = apply_skip(p, tr, 0.f, 1.f);
        if (p.stats) skip_stats_add(p, p.stats, k, has, fell, box_len, max(tr.ray.hi - tr.ray.lo, 0));
    }
    chunk_thread_ray(tr, k, p.K);

    float acc = 0.f;
    int first = INT_MAX, last = -1;  // non-empty extent of this thread's chunk
    float* cacc = smem + tid;  // MULTI: per-thread class accumulators, stride NT
    // MULTI: the samples of one class along a ray come in runs (label maps
    // are piecewise constant), so a run is summed in a register and added to
    // its class accumulator when the class changes, not one shared-memory
    // read-modify-write per sample.
    int run_cls = -1;
    float run = 0.f;
    if (MULTI) {
        for (int c = 0; c < p.C; ++c) cacc[c * NT] = 0.f;
    }
    // One sample's terms, in sample order.
    auto take = [&](int s, float x, float y, float z, const Cell& cell) {
        const float val = cell_value(cell);
        acc += val;
        if (p.out_extent) {
            const bool nz = (cell.v000 != 0.f) | (cell.v001 != 0.f) | (cell.v010 != 0.f) | (cell.v011 != 0.f) |
                            (cell.v100 != 0.f) | (cell.v101 != 0.f) | (cell.v110 != 0.f) | (cell.v111 != 0.f);
            if (nz) {
                first = min(first, s);
                last = s;
            }
        }
        if (MULTI) {
            int cls;
            if constexpr (QUAD == kLayoutQuadLab) {
                cls = cell.cls;
            } else {
                cls = nearest_label(p.lab, p.lab_dtype, p.D, p.H, p.W, x, y, z);
            }
            if (cls != run_cls) {
                if ((unsigned)run_cls < (unsigned)p.C) cacc[run_cls * NT] += run;
                run_cls = cls;
                run = 0.f;
            }
            run += val;
        }
    };
    // Quad layout: two samples per iteration, both cells loaded before either
    // is used, so two gathers per thread are in flight (label gathers: 3.88
    // against 4.28 ms at 512 x 512 x 400, 32 poses x 256^2, 8 channels; one
    // channel 2.12 against 2.13). The labelled layout keeps one sample per
    // iteration and trades registers for occupancy instead (2.88 ms, against
    // 3.31 paired), and so does the volume layout, whose one-pose forward is
    // DRAM-bound and lost resident CTAs to the pair's registers (64 against
    // 56; 200^2 x 500 samples: 74 against 64 us per graph replay).
    // Positions in float32, p0 + t * d with one rounding: the image is within
    // 1e-6 of the float64 oracle at 512^3 and the loop stays near 56
    // registers (fixed-point positions, which the adjoint uses, measured 28 %
    // slower here: 2.75 against 2.14 ms at 512^3 x 32 x 256^2).
    int s = tr.s0;
    if constexpr (QUAD == kLayoutQuad) {
        for (; s + 1 < tr.s1; s += 2) {
            const float ta = (float)s * p.inv_s, tb = (float)(s + 1) * p.inv_s;
            const float xa = fmaf(ta, tr.ray.dx, tr.ray.p0x), xb = fmaf(tb, tr.ray.dx, tr.ray.p0x);
            const float ya = fmaf(ta, tr.ray.dy, tr.ray.p0y), yb = fmaf(tb, tr.ray.dy, tr.ray.p0y);
            const float za = fmaf(ta, tr.ray.dz, tr.ray.p0z), zb = fmaf(tb, tr.ray.dz, tr.ray.p0z);
            Cell ca, cb;
            fetch_cell<VT, QUAD>(p, xa, ya, za, ca);
            fetch_cell<VT, QUAD>(p, xb, yb, zb, cb);
            take(s, xa, ya, za, ca);
            take(s + 1, xb, yb, zb, cb);
        }
    }
    for (; s < tr.s1; ++s) {
        const float t = (float)s * p.inv_s;
        const float x = fmaf(t, tr.ray.dx, tr.ray.p0x);
        const float y = fmaf(t, tr.ray.dy, tr.ray.p0y);
        const float z = fmaf(t, tr.ray.dz, tr.ray.p0z);
        Cell cell;
        fetch_cell<VT, QUAD>(p, x, y, z, cell);
        take(s, x, y, z, cell);
    }
    if (MULTI && (unsigned)run_cls < (unsigned)p.C) cacc[run_cls * NT] += run;

    // Sum the K chunk partials of each ray in a fixed order.
    float* red = smem + (MULTI ? (size_t)p.C * NT : 0);
    red[tid] = acc;
    if (p.out_extent) {
        // Non-empty extent across the K chunks (stored after the partials).
        int* ext = reinterpret_cast<int*>(red + NT);
        ext[tid] = first;
        ext[NT + tid] = last;
    }
    __syncthreads();
    if (p.out_extent && k == 0 && n >= 0) {
        const int* ext = reinterpret_cast<const int*>(red + NT);
        int f = ext[r], l = ext[NT + r];
        for (int j = 1; j < p.K; ++j) {
            f = min(f, ext[r + j * R]);
            l = max(l, ext[NT + r + j * R]);
        }
        const bool any = l >= 0;
        p.out_extent[tr.bn * 2 + 0] = any ? (float)f * p.inv_s : 1.f;
        p.out_extent[tr.bn * 2 + 1] = any ? (float)l * p.inv_s : 0.f;
    }
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

// Register budget of the forward per instantiation, set for occupancy: the
// loop is latency-bound, and more resident warps pay until spills cost more
// (kernel alone, 512 x 512 x 400 f32 / bf16, 32 poses x 256^2, 800 samples):
// f32 quad, one channel: 2.02 ms at 48 registers (10 CTAs of 128 per SM)
// against 2.10 at 56 and 2.41 at 40; f32 quad, 8 channels with label
// gathers: 3.77 at 40 against 3.81 at 48 and 3.93 at 64; labelled quad
// (bf16, 8 channels): 2.88 at 40 against 2.99 at 48 and 3.18 at 52; the
// volume layout: 3.59 at 64 against 3.83 at 48. Others keep 64 (two CTAs of
// 512 threads per SM).
template <typename VT, bool MULTI, int QUAD>
struct FwdRegs {
    static constexpr int value = QUAD == kLayoutQuadLab ? 40
                                 : (QUAD == kLayoutQuad && std::is_same<VT, float>::value) ? (MULTI ? 40 : 48)
                                                                                            : 64;
};

template <typename VT, typename OT, bool MULTI, int SKIP, int QUAD>
__global__ void __maxnreg__((FwdRegs<VT, MULTI, QUAD>::value)) raymarch_fwd_kernel(const MarchParams p) {
    fwd_body<VT, OT, MULTI, SKIP, QUAD>(p, blockIdx.x % p.tm.tiles, blockIdx.x / p.tm.tiles);
}

// ===================================================================== adjoint
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-thread adjoint accumulators. The pose partial of a ray is
//   dL/dM_ij = sum_s g_s dv_s,i [q_s, 1]_j,  q_s = src + t_s e,
// which this thread keeps as two 3-vectors, G = sum_s g_s dv_s and
// Gt = sum_s g_s dv_s t_s (6 multiply-adds per sample instead of 12 plus the
// position q_s), and expands once per ray: dL/dM_ij = G_i src_j + Gt_i e_j for
// j < 3, dL/dM_i3 = G_i (pose_terms).
struct AdjAcc {
    float G[3], Gt[3];
    float gsx, gsy, gsz, gtx, gty, gtz, gst;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int j = 0; j < 3; ++j) G[j] = Gt[j] = 0.f;
        gsx = gsy = gsz = gtx = gty = gtz = gst = 0.f;
    }
    __device__ __forceinline__ void pose_terms(float sx, float sy, float sz, float ex, float ey, float ez,
                                               float (&a)[12]) const {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            a[4 * i + 0] = fmaf(Gt[i], ex, G[i] * sx);
            a[4 * i + 1] = fmaf(Gt[i], ey, G[i] * sy);
            a[4 * i + 2] = fmaf(Gt[i], ez, G[i] * sz);
            a[4 * i + 3] = G[i];
        }
    }
};

// Volume-gradient scatter straight to global memory: one atomic per tap.
struct DirectScatter {
    float* __restrict__ gvol;
    int D, H, W;
    __device__ __forceinline__ void operator()(int idx_unused, int ix, int iy, int iz, float g00, float g01,
                                               float g10, float g11, float wx0, float wx1) const {
        (void)idx_unused;
        const int HW = H * W;
        const int base = (iz * H + iy) * W + ix;
        if ((unsigned)ix < (unsigned)(W - 1) && (unsigned)iy < (unsigned)(H - 1) && (unsigned)iz < (unsigned)(D - 1)) {
            atomicAdd(gvol + base, g00 * wx0);
            atomicAdd(gvol + base + 1, g00 * wx1);
            atomicAdd(gvol + base + W, g01 * wx0);
            atomicAdd(gvol + base + W + 1, g01 * wx1);
            atomicAdd(gvol + base + HW, g10 * wx0);
            atomicAdd(gvol + base + HW + 1, g10 * wx1);
            atomicAdd(gvol + base + HW + W, g11 * wx0);
            atomicAdd(gvol + base + HW + W + 1, g11 * wx1);
        } else {
            const bool x0 = (unsigned)ix < (unsigned)W, x1 = (unsigned)(ix + 1) < (unsigned)W;
            const bool y0 = (unsigned)iy < (unsigned)H, y1 = (unsigned)(iy + 1) < (unsigned)H;
            const bool z0 = (unsigned)iz < (unsigned)D, z1 = (unsigned)(iz + 1) < (unsigned)D;
            if (z0 && y0 && x0) atomicAdd(gvol + base, g00 * wx0);
            if (z0 && y0 && x1) atomicAdd(gvol + base + 1, g00 * wx1);
            if (z0 && y1 && x0) atomicAdd(gvol + base + W, g01 * wx0);
            if (z0 && y1 && x1) atomicAdd(gvol + base + W + 1, g01 * wx1);
            if (z1 && y0 && x0) atomicAdd(gvol + base + HW, g10 * wx0);
            if (z1 && y0 && x1) atomicAdd(gvol + base + HW + 1, g10 * wx1);
            if (z1 && y1 && x0) atomicAdd(gvol + base + HW + W, g11 * wx0);
            if (z1 && y1 && x1) atomicAdd(gvol + base + HW + W + 1, g11 * wx1);
        }
    }
};

// Volume-gradient scatter into a shared-memory brick covering the box
// [x0, x0 + nx) x [y0, y0 + ny) x [z0, z0 + nz), which contains every
// in-volume corner the current slab can touch (shared-memory atomics).
struct BrickScatter {
    float* acc;
    int D, H, W;
    int x0, y0, z0, nx, ny;
    __device__ __forceinline__ void operator()(int, int ix, int iy, int iz, float g00, float g01, float g10,
                                               float g11, float wx0, float wx1) const {
        const int lx = ix - x0, ly = iy - y0, lz = iz - z0;
        const int nxy = nx * ny;
        const int base = (lz * ny + ly) * nx + lx;
        const bool x0ok = (unsigned)ix < (unsigned)W, x1ok = (unsigned)(ix + 1) < (unsigned)W;
        const bool y0ok = (unsigned)iy < (unsigned)H, y1ok = (unsigned)(iy + 1) < (unsigned)H;
        const bool z0ok = (unsigned)iz < (unsigned)D, z1ok = (unsigned)(iz + 1) < (unsigned)D;
        if (z0ok && y0ok && x0ok) atomicAdd(acc + base, g00 * wx0);
        if (z0ok && y0ok && x1ok) atomicAdd(acc + base + 1, g00 * wx1);
        if (z0ok && y1ok && x0ok) atomicAdd(acc + base + nx, g01 * wx0);
        if (z0ok && y1ok && x1ok) atomicAdd(acc + base + nx + 1, g01 * wx1);
        if (z1ok && y0ok && x0ok) atomicAdd(acc + base + nxy, g10 * wx0);
        if (z1ok && y0ok && x1ok) atomicAdd(acc + base + nxy + 1, g10 * wx1);
        if (z1ok && y1ok && x0ok) atomicAdd(acc + base + nxy + nx, g11 * wx0);
        if (z1ok && y1ok && x1ok) atomicAdd(acc + base + nxy + nx + 1, g11 * wx1);
    }
};

// Volume-gradient scatter into the quad-layout gradient: the eight corner
// contributions of a sample are two 16-byte vector reductions (planes z0 and
// z0 + 1) at the sample's quad cell; ndrr_quad.cu folds the quad gradient
// back into the volume's layout afterwards. Indices come clamped into the
// padded extent, so no bounds checks are needed.
struct QuadScatter {
    float* __restrict__ gq;
    QuadGeom g;
    __device__ __forceinline__ void operator()(int, int ix, int iy, int iz, float g00, float g01, float g10,
                                               float g11, float wx0, float wx1) const {
        const int qi = ((iz + 2) * g.qy + (iy + 2)) * g.qx + (ix + 2);
        float* a = gq + (size_t)qi * 4;
        float* b = a + (size_t)g.plane * 4;
        // No "memory" clobber: nothing in the adjoint reads the gradient, so
        // the volume loads of later samples may be scheduled above these.
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(g00 * wx0), "f"(g00 * wx1),
                     "f"(g01 * wx0), "f"(g01 * wx1));
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(b), "f"(g10 * wx0), "f"(g10 * wx1),
                     "f"(g11 * wx0), "f"(g11 * wx1));
    }
};

// The same scatter with warp aggregation: the lanes of a warp that scatter
// into the same quad cell in the same step are found with __match_any_sync;
// the lowest such lane takes the second one's six factors by shuffle and
// issues the pair's reductions once, the second lane issues none (groups of
// three or more: the others reduce on their own). Among the 8 x 4 rays of a
// warp about 1.46 lanes share a cell on average at the benchmark's geometry
// (512^3 at 0.8 mm, 256^2 detector at 1.2 mm, 800 samples).
struct QuadScatterWarp {
    float* __restrict__ gq;
    QuadGeom g;
    __device__ __forceinline__ void operator()(int, int ix, int iy, int iz, float g00, float g01, float g10,
                                               float g11, float wx0, float wx1) const {
        const int qi = ((iz + 2) * g.qy + (iy + 2)) * g.qx + (ix + 2);
        const unsigned mask = __activemask();
        const int lane = threadIdx.x & 31;
        const unsigned peers = __match_any_sync(mask, qi);
        const int leader = __ffs(peers) - 1;
        const unsigned rest = peers & (peers - 1u);
        const int partner = rest ? __ffs(rest) - 1 : leader;
        const int src = lane == leader ? partner : lane;
        const float p00 = __shfl_sync(mask, g00, src), p01 = __shfl_sync(mask, g01, src);
        const float p10 = __shfl_sync(mask, g10, src), p11 = __shfl_sync(mask, g11, src);
        const float px0 = __shfl_sync(mask, wx0, src), px1 = __shfl_sync(mask, wx1, src);
        if (lane == partner && partner != leader) return;  // the leader issues this lane's terms
        float a0 = g00 * wx0, a1 = g00 * wx1, a2 = g01 * wx0, a3 = g01 * wx1;
        float b0 = g10 * wx0, b1 = g10 * wx1, b2 = g11 * wx0, b3 = g11 * wx1;
        if (lane == leader && partner != leader) {
            a0 += p00 * px0;
            a1 += p00 * px1;
            a2 += p01 * px0;
            a3 += p01 * px1;
            b0 += p10 * px0;
            b1 += p10 * px1;
            b2 += p11 * px0;
            b3 += p11 * px1;
        }
        float* a = gq + (size_t)qi * 4;
        float* b = a + (size_t)g.plane * 4;
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(a0), "f"(a1), "f"(a2), "f"(a3));
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(b), "f"(b0), "f"(b1), "f"(b2), "f"(b3));
    }
};

// Upstream gradient of one sample: the ray's own for one channel, else the
// one of the sample's label channel, with out-of-range labels masked like
// the forward drops them (_fused.py:233-237).
__device__ __forceinline__ float class_go(const MarchParams& p, int b, const ThreadRay& tr, int cls) {
    return ((unsigned)cls < (unsigned)p.C) ? ld_any_f(p.go, p.go_dtype, ((size_t)b * p.C + cls) * p.N + tr.n) : 0.f;
}

template <bool MULTI>
__device__ __forceinline__ float sample_go(const MarchParams& p, int b, const ThreadRay& tr, float go_ray,
                                           const FixPos& P) {
    if (!MULTI) return go_ray;
    return class_go(p, b, tr, nearest_label_fix(p.lab, p.lab_dtype, p.D, p.H, p.W, P));
}

// Adjoint terms of one sample whose cell is loaded.
template <bool GVOL, bool GCAM, typename Scatter>
__device__ __forceinline__ void adjoint_accumulate(const float (&m)[12], const ThreadRay& tr, float t, float gg,
                                                   const Cell& cell, AdjAcc& A, const Scatter& scatter);

// Adjoint of samples [s0, s1) of one ray (reference _fused.py:230-298).
// Samples go in pairs: both pairs' loads are issued before either's
// reductions, so two gathers per thread are in flight. The accumulation
// order is the sample order either way.
template <typename VT, bool MULTI, bool GVOL, bool GCAM, typename Scatter, int QUAD = kLayoutVolume>
__device__ __forceinline__ void adjoint_samples(const MarchParams& p, const float (&m)[12], const ThreadRay& tr,
                                                int b, int s0, int s1, float go_ray, AdjAcc& A,
                                                const Scatter& scatter) {
    if (!MULTI && go_ray == 0.f) return;  // every term is proportional to go
    // Each sample's position is formed from its index (f0 + s * step), not
    // stepped from the previous one: stepping chains every load address to
    // the last iteration's 64-bit add and measured 4.1 against 2.9 ms for the
    // pose adjoint at 512^3 x 32 x 256^2; independent positions let the loads
    // of later samples issue early, as with float positions.
    int s = s0;
    if constexpr (QUAD == kLayoutQuadLab) {
        // the class of a sample arrives with its corners: fetch, then route
        for (; s + 1 < s1; s += 2) {
            const float ta = (float)s * p.inv_s, tb = (float)(s + 1) * p.inv_s;
            const FixPos Pa = fix_at(tr, s), Pb = fix_at(tr, s + 1);
            Cell ca, cb;
            fetch_cell<VT, QUAD>(p, Pa, ca);
            fetch_cell<VT, QUAD>(p, Pb, cb);
            const float ga = MULTI ? class_go(p, b, tr, ca.cls) : go_ray;
            const float gb = MULTI ? class_go(p, b, tr, cb.cls) : go_ray;
            if (ga != 0.f) adjoint_accumulate<GVOL, GCAM>(m, tr, ta, ga, ca, A, scatter);
            if (gb != 0.f) adjoint_accumulate<GVOL, GCAM>(m, tr, tb, gb, cb, A, scatter);
        }
        if (s < s1) {
            const float t = (float)s * p.inv_s;
            Cell cell;
            fetch_cell<VT, QUAD>(p, fix_at(tr, s), cell);
            const float gg = MULTI ? class_go(p, b, tr, cell.cls) : go_ray;
            if (gg != 0.f) adjoint_accumulate<GVOL, GCAM>(m, tr, t, gg, cell, A, scatter);
        }
        return;
    }
    // Samples outside [glo, ghi) have eight zero corners (the window of an
    // exact skip): no pose terms, so their cells are not loaded, while their
    // volume-gradient terms (which need no corner values) are scattered.
    for (; s + 1 < s1; s += 2) {
        const float ta = (float)s * p.inv_s, tb = (float)(s + 1) * p.inv_s;
        const FixPos Pa = fix_at(tr, s), Pb = fix_at(tr, s + 1);
        const float ga = sample_go<MULTI>(p, b, tr, go_ray, Pa);
        const float gb = sample_go<MULTI>(p, b, tr, go_ray, Pb);
        Cell ca, cb;
        if (MULTI || (s >= tr.glo && s < tr.ghi))
            fetch_cell<VT, QUAD>(p, Pa, ca);
        else
            zero_cell(p, Pa, ca);
        if (MULTI || (s + 1 >= tr.glo && s + 1 < tr.ghi))
            fetch_cell<VT, QUAD>(p, Pb, cb);
        else
            zero_cell(p, Pb, cb);
        if (ga != 0.f) adjoint_accumulate<GVOL, GCAM>(m, tr, ta, ga, ca, A, scatter);
        if (gb != 0.f) adjoint_accumulate<GVOL, GCAM>(m, tr, tb, gb, cb, A, scatter);
    }
    if (s < s1) {
        const float t = (float)s * p.inv_s;
        const FixPos Pa = fix_at(tr, s);
        const float gg = sample_go<MULTI>(p, b, tr, go_ray, Pa);
        if (gg != 0.f) {
            Cell cell;
            if (MULTI || (s >= tr.glo && s < tr.ghi))
                fetch_cell<VT, QUAD>(p, Pa, cell);
            else
                zero_cell(p, Pa, cell);
            adjoint_accumulate<GVOL, GCAM>(m, tr, t, gg, cell, A, scatter);
        }
    }
}

template <bool GVOL, bool GCAM, typename Scatter>
__device__ __forceinline__ void adjoint_accumulate(const float (&m)[12], const ThreadRay& tr, float t, float gg,
                                                   const Cell& cell, AdjAcc& A, const Scatter& scatter) {
    const float g = gg * tr.stepv;
    float dvx, dvy, dvz;
    cell_grad(cell, dvx, dvy, dvz);
    const float gx = g * dvx, gy = g * dvy, gz = g * dvz;
    A.G[0] += gx;
    A.G[1] += gy;
    A.G[2] += gz;
    A.Gt[0] = fmaf(gx, t, A.Gt[0]);
    A.Gt[1] = fmaf(gy, t, A.Gt[1]);
    A.Gt[2] = fmaf(gz, t, A.Gt[2]);
    if (GCAM) {
        // Chain to camera space: gq = M[:, :3]^T gpos.
        const float gqx = m[0] * gx + m[4] * gy + m[8] * gz;
        const float gqy = m[1] * gx + m[5] * gy + m[9] * gz;
        const float gqz = m[2] * gx + m[6] * gy + m[10] * gz;
        const float omt = 1.f - t;
        A.gsx = fmaf(omt, gqx, A.gsx);
        A.gsy = fmaf(omt, gqy, A.gsy);
        A.gsz = fmaf(omt, gqz, A.gsz);
        A.gtx = fmaf(t, gqx, A.gtx);
        A.gty = fmaf(t, gqy, A.gty);
        A.gtz = fmaf(t, gqz, A.gtz);
        A.gst = fmaf(gg, cell_value(cell), A.gst);
    }
    if (GVOL) {
        const float wy0 = 1.f - cell.fy, wz0 = 1.f - cell.fz;
        scatter(0, cell.ix, cell.iy, cell.iz, g * wz0 * wy0, g * wz0 * cell.fy, g * cell.fz * wy0,
                g * cell.fz * cell.fy, 1.f - cell.fx, cell.fx);
    }
}

// CTA epilogue shared by the adjoint kernels: fixed-order reduction of the
// pose partials into `partials[slot]`, and the per-ray camera
// gradients (summing the K sample chunks of each ray in order).
template <bool GCAM>
__device__ __forceinline__ void adjoint_epilogue(const MarchParams& p, const size_t slot, const ThreadRay& tr,
                                                 const AdjAcc& A,
                                                 float* smem, int R, int NT, int r, int k) {
    const int tid = threadIdx.x;
    const bool shared_src = GCAM && !p.src_per_ray;
    const int nwarps = NT >> 5;
    const int warp = tid >> 5, lane = tid & 31;
    float* wred = smem;  // [nwarps][kPartialStride]
    float a[12];
    A.pose_terms(tr.sx, tr.sy, tr.sz, tr.ex, tr.ey, tr.ez, a);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        const float v = warp_sum(a[j]);
        if (lane == 0) wred[warp * kPartialStride + j] = v;
    }
    if (shared_src) {
        const float v0 = warp_sum(A.gsx), v1 = warp_sum(A.gsy), v2 = warp_sum(A.gsz);
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
        p.partials[slot * kPartialStride + tid] = sum;
    }
    if (GCAM) {
        __syncthreads();
        float* cr = smem;  // [7][NT]
        cr[0 * NT + tid] = A.gtx;
        cr[1 * NT + tid] = A.gty;
        cr[2 * NT + tid] = A.gtz;
        cr[3 * NT + tid] = A.gst;
        cr[4 * NT + tid] = A.gsx;
        cr[5 * NT + tid] = A.gsy;
        cr[6 * NT + tid] = A.gsz;
        __syncthreads();
        if (k == 0 && tr.n >= 0) {
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

// Adjoint with direct global atomics for the volume gradient.
// SKIP (only with GVOL false, see apply_skip): 0 none, 1 occupancy.
// Volume slab of the slab-ordered adjoint: only samples whose scatter cell
// along `axis` (shifted by 2, see cell_index_shifted) lies in [c0, c1).
struct SlabCut {
    int axis;
    int c0, c1;
};

// Cell index of the quad scatter along one axis at sample s (fix_cell's
// clamped integer part), shifted by 2 into [0, dim + 2].
__device__ __forceinline__ int cell_index_shifted(const ThreadRay& tr, int axis, int s, int dim) {
    const long long f0 = axis == 0 ? tr.f0.x : (axis == 1 ? tr.f0.y : tr.f0.z);
    const long long fd = axis == 0 ? tr.fd.x : (axis == 1 ? tr.fd.y : tr.fd.z);
    return min(max(fix_floor(f0 + (long long)s * fd), -2), dim) + 2;
}

// First s in [lo, hi) whose cell index along the cut's axis is >= c (index
// non-decreasing in s) or < c (non-increasing); hi when there is none. The
// index is monotonic in s (exact integer positions), so a binary search over
// the same per-sample computation the march uses finds the boundary.
__device__ __forceinline__ int slab_bound(const ThreadRay& tr, int axis, int dim, int lo, int hi, int c,
                                          bool increasing) {
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        const int i = cell_index_shifted(tr, axis, mid, dim);
        if (increasing ? (i >= c) : (i < c))
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// Restrict a ray's window to the samples of one slab.
__device__ __forceinline__ void restrict_to_slab(const MarchParams& p, ThreadRay& tr, const SlabCut& cut) {
    Ray& r = tr.ray;
    if (r.lo >= r.hi) return;
    const int dim = cut.axis == 0 ? p.W : (cut.axis == 1 ? p.H : p.D);
    const long long d = cut.axis == 0 ? tr.fd.x : (cut.axis == 1 ? tr.fd.y : tr.fd.z);
    int a, e;
    if (d > 0) {
        a = slab_bound(tr, cut.axis, dim, r.lo, r.hi, cut.c0, true);
        e = slab_bound(tr, cut.axis, dim, a, r.hi, cut.c1, true);
    } else if (d < 0) {
        a = slab_bound(tr, cut.axis, dim, r.lo, r.hi, cut.c1, false);
        e = slab_bound(tr, cut.axis, dim, a, r.hi, cut.c0, false);
    } else {
        const int i = cell_index_shifted(tr, cut.axis, r.lo, dim);
        const bool in = i >= cut.c0 && i < cut.c1;
        a = r.lo;
        e = in ? r.hi : r.lo;
    }
    r.lo = a;
    r.hi = e;
}

template <typename VT, bool MULTI, bool GVOL, bool GCAM, int SKIP, int QUAD = kLayoutVolume, bool SLAB = false,
          bool WARP_AGG = false>
__device__ __forceinline__ void bwd_body(const MarchParams& p, const int tile, const int b, const size_t slot,
                                         const SlabCut cut = SlabCut{0, 0, 0}) {
    extern __shared__ float smem[];
    const int R = p.tw * p.th;
    const int NT = R * p.K;
    const int tid = threadIdx.x;
    const int r = tid % R, k = tid / R;
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, r);

    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
    ThreadRay tr;
    init_thread_ray(p, m, b, n, tr);
    if (!GVOL && SKIP != 0) {
        // Skipped samples have eight zero corners: no pose or camera terms.
        apply_skip(p, tr, 0.f, 1.f);
    }
    if constexpr (SLAB) {
        restrict_to_slab(p, tr, cut);
        if (!MULTI && p.gwin && n >= 0) {
            const int2 w = __ldg(reinterpret_cast<const int2*>(p.gwin) + tr.bn);
            tr.glo = w.x;
            tr.ghi = w.y;
        }
    }
    chunk_thread_ray(tr, k, p.K);
    float go_ray = 0.f;
    if (!MULTI && n >= 0) go_ray = ld_any_f(p.go, p.go_dtype, tr.bn);

    AdjAcc A;
    A.zero();
    if constexpr (QUAD != kLayoutVolume && WARP_AGG) {
        const QuadScatterWarp sc{p.gquad, p.qg};
        adjoint_samples<VT, MULTI, GVOL, GCAM, QuadScatterWarp, QUAD>(p, m, tr, b, tr.s0, tr.s1, go_ray, A, sc);
    } else if constexpr (QUAD != kLayoutVolume) {
        const QuadScatter sc{p.gquad, p.qg};
        adjoint_samples<VT, MULTI, GVOL, GCAM, QuadScatter, QUAD>(p, m, tr, b, tr.s0, tr.s1, go_ray, A, sc);
    } else {
        const DirectScatter sc{p.gvol, p.D, p.H, p.W};
        adjoint_samples<VT, MULTI, GVOL, GCAM>(p, m, tr, b, tr.s0, tr.s1, go_ray, A, sc);
    }
    adjoint_epilogue<GCAM>(p, slot, tr, A, smem, R, NT, r, k);
}

// Register budget of the adjoint: 128 (one CTA of 512 threads per SM), but
// 56 for the one-channel pose-only adjoint of an f32 quad volume without an
// in-kernel skip, where occupancy pays: 2.80 against 2.86 ms at 70
// registers (512^3, 32 poses x 256^2, 800 samples, kernel alone; 64
// measured 3.16).
template <typename VT, bool MULTI, bool GVOL, bool GCAM, int SKIP, int QUAD>
struct BwdRegs {
    static constexpr int value =
        (!MULTI && !GVOL && !GCAM && SKIP == 0 && QUAD == kLayoutQuad && std::is_same<VT, float>::value) ? 56
                                                                                                          : 128;
};

template <typename VT, bool MULTI, bool GVOL, bool GCAM, int SKIP, int QUAD>
__global__ void __maxnreg__((BwdRegs<VT, MULTI, GVOL, GCAM, SKIP, QUAD>::value)) raymarch_bwd_kernel(const MarchParams p) {
    bwd_body<VT, MULTI, GVOL, GCAM, SKIP, QUAD>(p, blockIdx.x % p.tm.tiles, blockIdx.x / p.tm.tiles, blockIdx.x);
}

// Block-wide min of (a0..a2, -b0..-b2): the union box of per-thread boxes.
// `sred` holds nwarps * 6 ints; the result lands in box[0..5] for every thread.
__device__ __forceinline__ void block_box(int (&lo)[3], int (&hi)[3], int* sred, int* box, int nwarps) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int v[6] = {lo[0], lo[1], lo[2], -hi[0], -hi[1], -hi[2]};
#pragma unroll
    for (int j = 0; j < 6; ++j) v[j] = __reduce_min_sync(0xffffffffu, v[j]);
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < 6; ++j) sred[warp * 6 + j] = v[j];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        int m = sred[threadIdx.x];
        for (int w = 1; w < nwarps; ++w) m = min(m, sred[w * 6 + threadIdx.x]);
        box[threadIdx.x] = m;
    }
    __syncthreads();
    lo[0] = box[0];
    lo[1] = box[1];
    lo[2] = box[2];
    hi[0] = -box[3];
    hi[1] = -box[4];
    hi[2] = -box[5];
}

__device__ __forceinline__ int floor_clamped(long long v, int lo, int hi) {
    return min(max(fix_floor(v), lo), hi);
}

// Adjoint with the volume gradient privatised per slab: the CTA's rays march
// in lockstep over sample slabs [sb, sb + L); for each slab the union of the
// rays' cell boxes (exact: positions are monotone in s, so the two slab ends
// bound every sample) is accumulated in shared memory and flushed to global
// memory with one coalesced atomic per touched voxel. Slabs whose box exceeds
// `cap` voxels fall back to direct atomics, and L adapts to keep boxes small.
// One thread per ray (sample_split = 1).
template <typename VT, bool MULTI, bool GCAM>
__global__ void __launch_bounds__(256, 2) raymarch_bwd_brick_kernel(const MarchParams p, int cap, int L0) {
    extern __shared__ float smem[];
    const int R = p.tw * p.th;
    const int NT = R;
    const int nwarps = NT >> 5;
    const int tid = threadIdx.x;
    const int tile = blockIdx.x % p.tm.tiles;
    const int b = blockIdx.x / p.tm.tiles;
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, tid);
    float* acc = smem;                                   // [cap] brick
    int* sred = reinterpret_cast<int*>(smem + cap);      // [nwarps * 6]
    int* box = sred + nwarps * 6;                        // [8]

    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
    ThreadRay tr;
    setup_thread_ray(p, m, b, n, 0, tr);
    float go_ray = 0.f;
    if (!MULTI && n >= 0) go_ray = ld_any_f(p.go, p.go_dtype, tr.bn);

    // Tile-wide sample range. Empty entries use (INT_MAX, -INT_MAX) so that
    // the negation inside block_box cannot overflow.
    int lo3[3], hi3[3];
    {
        const bool any = tr.s0 < tr.s1;
        lo3[0] = any ? tr.s0 : INT_MAX;
        hi3[0] = any ? tr.s1 : -INT_MAX;
        lo3[1] = lo3[2] = INT_MAX;
        hi3[1] = hi3[2] = -INT_MAX;
        block_box(lo3, hi3, sred, box, nwarps);
    }
    const int smin = lo3[0], smax = hi3[0];

    AdjAcc A;
    A.zero();
    int L = L0;
    for (int sb = smin; sb < smax;) {
        const int se = min(sb + L, smax);
        const int a = max(tr.s0, sb), e = min(tr.s1, se);
        lo3[0] = lo3[1] = lo3[2] = INT_MAX;
        hi3[0] = hi3[1] = hi3[2] = -INT_MAX;
        if (a < e) {
            const FixPos Pa = fix_at(tr, a), Pe = fix_at(tr, e - 1);
            const int xa = floor_clamped(Pa.x, -2, p.W), xe = floor_clamped(Pe.x, -2, p.W);
            const int ya = floor_clamped(Pa.y, -2, p.H), ye = floor_clamped(Pe.y, -2, p.H);
            const int za = floor_clamped(Pa.z, -2, p.D), ze = floor_clamped(Pe.z, -2, p.D);
            // corners span [floor, floor + 1], clipped to the volume
            int l0 = max(min(xa, xe), 0), h0 = min(max(xa, xe) + 1, p.W - 1);
            int l1 = max(min(ya, ye), 0), h1 = min(max(ya, ye) + 1, p.H - 1);
            int l2 = max(min(za, ze), 0), h2 = min(max(za, ze) + 1, p.D - 1);
            if (l0 <= h0 && l1 <= h1 && l2 <= h2) {
                lo3[0] = l0; lo3[1] = l1; lo3[2] = l2;
                hi3[0] = h0; hi3[1] = h1; hi3[2] = h2;
            }
        }
        block_box(lo3, hi3, sred, box, nwarps);
        const bool empty = lo3[0] > hi3[0];
        const int nx = empty ? 0 : hi3[0] - lo3[0] + 1;
        const int ny = empty ? 0 : hi3[1] - lo3[1] + 1;
        const int nz = empty ? 0 : hi3[2] - lo3[2] + 1;
        const long long nvox = (long long)nx * ny * nz;
        const bool use_brick = nvox > 0 && nvox <= cap;
        if (use_brick) {
            float4* a4 = reinterpret_cast<float4*>(acc);
            const int n4 = (int)(nvox >> 2);
            for (int i = tid; i < n4; i += NT) a4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int i = (n4 << 2) + tid; i < (int)nvox; i += NT) acc[i] = 0.f;
            __syncthreads();
            const BrickScatter sc{acc, p.D, p.H, p.W, lo3[0], lo3[1], lo3[2], nx, ny};
            adjoint_samples<VT, MULTI, true, GCAM>(p, m, tr, b, a, e, go_ray, A, sc);
            __syncthreads();
            // Flush: each warp takes whole rows so lanes write consecutive x.
            const int warp = tid >> 5, lane = tid & 31;
            const int rows = ny * nz;
            for (int row = warp; row < rows; row += nwarps) {
                const int ly = row % ny, lz = row / ny;
                float* g = p.gvol + ((size_t)(lo3[2] + lz) * p.H + (lo3[1] + ly)) * p.W + lo3[0];
                const float* s = acc + row * nx;
                for (int lx = lane; lx < nx; lx += 32) {
                    const float v = s[lx];
                    if (v != 0.f) atomicAdd(g + lx, v);
                }
            }
            if (nvox * 4 < cap) L = min(L * 2, 256);
        } else {
            const DirectScatter sc{p.gvol, p.D, p.H, p.W};
            adjoint_samples<VT, MULTI, true, GCAM>(p, m, tr, b, a, e, go_ray, A, sc);
            if (nvox > cap) L = max(L >> 1, 2);
        }
        sb = se;
    }
    adjoint_epilogue<GCAM>(p, blockIdx.x, tr, A, smem, R, NT, tid, 0);
}

// Per-pose sum of the per-tile partials in a fixed order. One CTA per pose.
cudaError_t launch_brick(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p, unsigned grid,
                         unsigned block, cudaStream_t st);
// Quad-layout instantiations live in their own translation units.
cudaError_t launch_fwd_quad(const MarchParams& p, int vol_dtype, bool multi, int skip, bool labeled, unsigned grid,
                            unsigned block, size_t smem, cudaStream_t st);
cudaError_t launch_bwd_quad(const MarchParams& p, int vol_dtype, bool multi, bool gvol, bool gcam, int skip,
                            bool labeled, unsigned grid, unsigned block, size_t smem, cudaStream_t st);
cudaError_t launch_quad_fold(const float* gquad, int D, int H, int W, float* gvol, bool overwrite, cudaStream_t st);
cudaError_t launch_quad_build(const void* vol, int dtype, int D, int H, int W, void* quad, cudaStream_t st);
cudaError_t launch_quad_build_labeled(const void* vol, int dtype, const void* lab, int lab_dtype, int C, int D, int H,
                                      int W, void* quad, cudaStream_t st);

MarchParams make_params(const ndrr_raymarch_args& a, const LaunchShape& ls);
cudaError_t launch_bwd_slab(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p,
                            cudaStream_t st);
cudaError_t launch_scatter_slab(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p0,
                                cudaStream_t st);
size_t fwd_base_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls);

template <typename Kern>
static cudaError_t launch_kernel(Kern kern, unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                                 const MarchParams& p) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const KernelEvents& ev = kernel_events();
    if (ev.start != nullptr) cudaEventRecord(ev.start, st);
    kern<<<grid, block, smem, st>>>(p);
    cudaError_t e = cudaGetLastError();
    if (ev.stop != nullptr && e == cudaSuccess) e = cudaEventRecord(ev.stop, st);
    return e;
}

}  // namespace ndrr
