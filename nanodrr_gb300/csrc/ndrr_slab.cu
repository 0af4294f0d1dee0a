// Slab-ordered adjoint with volume gradient (quad layout).
//
// The volume-gradient adjoint is bound by read-modify-write traffic: each
// pose's rays sweep the whole quad gradient (16 B per cell-plane corner
// quad, 4x the volume), and by the time the next pose sweeps the same
// region the previous sweep's lines have left the 126 MB L2, so every pose
// pays a DRAM read and write of everything it touches. Here the volume is cut
// into slabs along one axis per pose (the axis the pose's rays run most
// nearly parallel to its planes, so that each ray crosses few slabs), each
// slab about 128 MB of quad gradient, and the work is ordered slab by slab across ALL
// poses: a work item is (slab, pose, detector tile), marching only the
// samples whose scatter cell lies in the slab. Items of one slab run
// together, so the slab's gradient (and volume) lines are reused from L2 by
// every pose before they are evicted.
//
// Determinism of the pose gradient: every item writes its CTA partial to a
// fixed slot (tile offset from a prefix sum + slab rank within the tile's
// slab range), and the per-pose sum runs over tiles and slabs in a fixed
// order, so gM does not depend on which CTA took which item when.
//
// Steps (one stream, no host synchronisation, capturable):
//   slab_plan_kernel     per (pose, tile): the pose's axis and the tile's
//                        slab range [k0, k1]; a histogram of items per slab
//   slab_scan_kernel     prefix sums: tile offsets of the partial slots and
//                        the start of each slab's items in the work list
//   slab_fill_kernel     the work list, grouped by slab
//   raymarch_bwd_slab_kernel  persistent CTAs take items from an atomic
//                        counter in list order
//   slab_pose_reduce_kernel   fixed-order per-pose sums of the partials
#include "ndrr_march.cuh"

namespace ndrr {

// Workspace layout, computed identically on the host (sizes) and passed to
// the kernels as pointers.
struct SlabParams {
    int Z[3];         // slab thickness in cells per axis (x, y, z)
    int ns[3];        // slabs per axis
    int base[3];      // first global slab id of each axis
    int* counters;    // [0] items, [1] work counter
    int* hist;        // [ns_total * kSortBuckets] items per (global slab, bucket), then cursors
    int* key;         // [B * tiles] bucket of each tile along its pose's sort axis
    int2* trange;     // [B * tiles] slab range of each tile (k0 > k1: none)
    int* count;       // [B * tiles] items of each tile
    int* offset;      // [B * tiles + 1] first partial slot of each tile
    int* axis;        // [B] slab axis of each pose
    int2* items;      // [max_items] (pose * tiles + tile, slab)
    float* partials;  // [max_items][kPartialStride]
    int ns_total;
    int BT;
};

// Quad-gradient bytes per slab. Measured at 512^3 x 32 poses (adjoint ms):
// 4 MiB 20.5, 8 MiB 20.5, 24 MiB 11.1, 48 MiB 9.8, 96 MiB 9.4, 192 MiB 10.2,
// 384 MiB 11.0, direct scatter 10.3-10.6: thin slabs multiply the work items
// (each ray is cut once per slab crossed), thick ones lose the L2 reuse.
// With the items of a slab ordered by bucket (below), the march kernel alone:
// 64 MiB 6.84, 96 MiB 6.59, 128 MiB 6.51, 160 MiB 6.54, 192 MiB 6.67, 256 MiB
// 7.03 ms (6.79 at 96 MiB before the ordering).
constexpr size_t kSlabTargetBytes = 128u << 20;  // default; args.slab_mib overrides

// Items of one slab are ordered by bucket along a second axis (the one of the
// two others that the pose's rays run least along, so a tile's rays stay
// within a band of it): the CTAs running at one time then work in a band of
// the slab instead of all of it, and the band's volume and gradient lines
// stay in L2 while every pose's rays through it are marched. The order
// changes no result (pose partials have fixed slots).
constexpr int kSortBuckets = 32;

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Host-side slab geometry: thickness per axis so that a slab of the quad
// gradient holds about the target bytes (at least one cell).
static void slab_geometry(const ndrr_raymarch_args& a, int Z[3], int ns[3]) {
    const long long target = a.slab_mib > 0 ? (long long)a.slab_mib << 20 : (long long)kSlabTargetBytes;
    const long long qx = a.W + 3, qy = a.H + 3, qz = a.D + 4;
    const long long plane[3] = {qz * qy * 16, qz * qx * 16, qy * qx * 16};  // bytes per unit thickness
    const int cells[3] = {a.W + 3, a.H + 3, a.D + 3};  // shifted cell indices 0 .. dim + 2
    for (int i = 0; i < 3; ++i) {
        Z[i] = (int)std::max<long long>(1, target / std::max<long long>(plane[i], 1));
        Z[i] = std::min(Z[i], cells[i]);
        ns[i] = (cells[i] + Z[i] - 1) / Z[i];
    }
}

struct SlabLayout {
    size_t counters, hist, key, trange, count, offset, axis, items, partials, total;
    long long max_items;
};

static SlabLayout slab_layout(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    int Z[3], ns[3];
    slab_geometry(a, Z, ns);
    const TileMap tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
    const long long BT = (long long)a.B * tm.tiles;
    const int ns_total = ns[0] + ns[1] + ns[2];
    const int ns_max = std::max(ns[0], std::max(ns[1], ns[2]));
    SlabLayout L;
    L.max_items = BT * ns_max;
    size_t o = 0;
    L.counters = o; o = align16(o + 4 * sizeof(int));
    L.hist = o;     o = align16(o + (size_t)ns_total * kSortBuckets * sizeof(int));
    L.key = o;      o = align16(o + (size_t)BT * sizeof(int));
    L.trange = o;   o = align16(o + (size_t)BT * sizeof(int2));
    L.count = o;    o = align16(o + (size_t)BT * sizeof(int));
    L.offset = o;   o = align16(o + (size_t)(BT + 1) * sizeof(int));
    L.axis = o;     o = align16(o + (size_t)a.B * sizeof(int));
    L.items = o;    o = align16(o + (size_t)L.max_items * sizeof(int2));
    L.partials = o; o = align16(o + (size_t)L.max_items * kPartialStride * sizeof(float));
    L.total = o;
    return L;
}

uint64_t slab_workspace_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    return slab_layout(a, ls).total;
}

// Slab axis of a pose: z, whose slabs are contiguous runs of planes of the
// quad gradient (planes are its outermost index), unless the camera's optical
// axis (third column of M) runs mostly along z; then the axis of its
// smaller x/y component. At 512^3 x 32 poses (rays mostly along y) the
// adjoint took 7.9 ms with z slabs for every pose, 9.3 ms with each pose's
// least-crossed axis (a mix of x and z slabs, so the gradient is swept once
// per axis) and 10.1 ms with x slabs for every pose.
__device__ __forceinline__ int pose_slab_axis(const float (&m)[12]) {
    const float ax = fabsf(m[2]), ay = fabsf(m[6]), az = fabsf(m[10]);
    if (az < fmaxf(ax, ay)) return 2;
    return ay < ax ? 1 : 0;
}

// The item-ordering axis of a pose: of the two axes other than its slab axis,
// the one its optical axis has the smaller component along.
__device__ __forceinline__ int pose_sort_axis(const float (&m)[12], int slab_axis) {
    const float c[3] = {fabsf(m[2]), fabsf(m[6]), fabsf(m[10])};
    const int a0 = slab_axis == 0 ? 1 : 0, a1 = slab_axis == 2 ? 1 : 2;
    return c[a1] < c[a0] ? a1 : a0;
}

// ---------------------------------------------------------------- planning
__global__ void __launch_bounds__(512) slab_plan_kernel(const MarchParams p, const SlabParams s) {
    __shared__ int red[4];
    const int R = p.tw * p.th;
    const int bt = blockIdx.x;
    const int b = bt / p.tm.tiles, tile = bt % p.tm.tiles;
    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
    const int axis = pose_slab_axis(m);
    const int sort_axis = pose_sort_axis(m, axis);
    if (threadIdx.x == 0) {
        red[0] = INT_MAX;
        red[1] = -1;
        red[2] = 0;  // sum of the rays' buckets along the sort axis
        red[3] = 0;  // rays counted
        if (tile == 0) s.axis[b] = axis;
    }
    __syncthreads();
    if ((int)threadIdx.x < R) {
        const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, threadIdx.x);
        ThreadRay tr;
        init_thread_ray(p, m, b, n, tr);
        if (n >= 0 && tr.ray.lo < tr.ray.hi) {
            const int dim = axis == 0 ? p.W : (axis == 1 ? p.H : p.D);
            const int i0 = cell_index_shifted(tr, axis, tr.ray.lo, dim);
            const int i1 = cell_index_shifted(tr, axis, tr.ray.hi - 1, dim);
            atomicMin(&red[0], min(i0, i1) / s.Z[axis]);
            atomicMax(&red[1], max(i0, i1) / s.Z[axis]);
            // bucket of the window's middle sample along the sort axis
            const int sdim = sort_axis == 0 ? p.W : (sort_axis == 1 ? p.H : p.D);
            const int im = cell_index_shifted(tr, sort_axis, (tr.ray.lo + tr.ray.hi - 1) >> 1, sdim);
            atomicAdd(&red[2], (int)(((long long)im * kSortBuckets) / (sdim + 3)));
            atomicAdd(&red[3], 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int k0 = red[0], k1 = red[1];
        if (k1 >= 0) {
            s.trange[bt] = make_int2(k0, k1);
            s.count[bt] = k1 - k0 + 1;
            const int key = min(kSortBuckets - 1, max(0, red[2] / max(red[3], 1)));
            s.key[bt] = key;
            for (int k = k0; k <= k1; ++k) atomicAdd(&s.hist[(s.base[axis] + k) * kSortBuckets + key], 1);
        } else {
            s.trange[bt] = make_int2(1, 0);
            s.count[bt] = 0;
        }
    }
}

// Exclusive scan of n ints in place (one CTA), returning the total.
__device__ int block_exclusive_scan(int* v, int n, int* sh) {
    const int T = blockDim.x, tid = threadIdx.x;
    const int per = (n + T - 1) / T;
    const int beg = min(n, tid * per), end = min(n, beg + per);
    int sum = 0;
    for (int i = beg; i < end; ++i) sum += v[i];
    sh[tid] = sum;
    __syncthreads();
    // Hillis-Steele over the per-thread sums
    for (int o = 1; o < T; o <<= 1) {
        const int x = tid >= o ? sh[tid - o] : 0;
        __syncthreads();
        sh[tid] += x;
        __syncthreads();
    }
    int run = sh[tid] - sum;  // exclusive prefix of this thread's chunk
    for (int i = beg; i < end; ++i) {
        const int c = v[i];
        v[i] = run;
        run += c;
    }
    const int total = sh[T - 1];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(1024) slab_scan_kernel(const SlabParams s) {
    __shared__ int sh[1024];
    // tile offsets: offset[bt] = sum of count over earlier tiles
    for (int i = threadIdx.x; i < s.BT; i += blockDim.x) s.offset[i] = s.count[i];
    __syncthreads();
    const int items = block_exclusive_scan(s.offset, s.BT, sh);
    if (threadIdx.x == 0) s.offset[s.BT] = items;
    // slab cursors: start of each slab's items in the list
    block_exclusive_scan(s.hist, s.ns_total * kSortBuckets, sh);
    if (threadIdx.x == 0) {
        s.counters[0] = items;
        s.counters[1] = 0;
    }
}

__global__ void __launch_bounds__(256) slab_fill_kernel(const SlabParams s, int tiles) {
    const int bt = blockIdx.x * blockDim.x + threadIdx.x;
    if (bt >= s.BT) return;
    const int2 r = s.trange[bt];
    if (r.x > r.y) return;
    const int axis = s.axis[bt / tiles];
    for (int k = r.x; k <= r.y; ++k) {
        const int pos = atomicAdd(&s.hist[(s.base[axis] + k) * kSortBuckets + s.key[bt]], 1);
        s.items[pos] = make_int2(bt, k);
    }
}

// ------------------------------------------------------------- the adjoint
template <typename VT, bool MULTI, bool WARP_AGG, int LAYOUT>
__global__ void __maxnreg__(96) raymarch_bwd_slab_kernel(const MarchParams p, const SlabParams s) {
    __shared__ int item_sh;
    const int total = s.counters[0];
    while (true) {
        __syncthreads();  // the previous item is done with item_sh and shared memory
        if (threadIdx.x == 0) item_sh = atomicAdd(&s.counters[1], 1);
        __syncthreads();
        const int item = item_sh;
        if (item >= total) break;
        const int2 it = s.items[item];
        const int bt = it.x, k = it.y;
        const int b = bt / p.tm.tiles, tile = bt % p.tm.tiles;
        const int axis = s.axis[b];
        // selected, not indexed: a run-time index into the by-value kernel
        // parameter would copy the parameter struct to local memory
        const int thick = axis == 0 ? s.Z[0] : (axis == 1 ? s.Z[1] : s.Z[2]);
        const SlabCut cut{axis, k * thick, (k + 1) * thick};
        const size_t slot = (size_t)s.offset[bt] + (size_t)(k - s.trange[bt].x);
        bwd_body<VT, MULTI, true, false, 0, LAYOUT, true, WARP_AGG>(p, tile, b, slot, cut);
    }
}

// Volume-gradient scatter of one (slab, pose, tile) item from sample
// positions alone: the split adjoint's second pass. The terms are those of
// adjoint_accumulate's scatter (go * step * trilinear weight per corner, two
// 16-byte reductions into the quad gradient per sample); the volume values
// and the pose terms, which need the gathers, come from the first pass.
__device__ __forceinline__ void scatter_body(const MarchParams& p, const int tile, const int b,
                                             const SlabCut cut) {
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, (int)threadIdx.x);
    if (n < 0) return;
    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
    ThreadRay tr;
    init_thread_ray(p, m, b, n, tr);
    restrict_to_slab(p, tr, cut);
    const float go = ld_any_f(p.go, p.go_dtype, tr.bn);
    if (go == 0.f) return;  // every term is proportional to go
    const float g = go * tr.stepv;
    const QuadScatter sc{p.gquad, p.qg};
    for (int s = tr.ray.lo; s < tr.ray.hi; ++s) {
        Cell c;
        fix_cell(fix_at(tr, s), p.D, p.H, p.W, c);
        const float wy0 = 1.f - c.fy, wz0 = 1.f - c.fz;
        sc(0, c.ix, c.iy, c.iz, g * wz0 * wy0, g * wz0 * c.fy, g * c.fz * wy0, g * c.fz * c.fy, 1.f - c.fx, c.fx);
    }
}

__global__ void __launch_bounds__(512) raymarch_scatter_slab_kernel(const MarchParams p, const SlabParams s) {
    __shared__ int item_sh;
    const int total = s.counters[0];
    while (true) {
        __syncthreads();  // every thread has read item_sh
        if (threadIdx.x == 0) item_sh = atomicAdd(&s.counters[1], 1);
        __syncthreads();
        const int item = item_sh;
        if (item >= total) break;
        const int2 it = s.items[item];
        const int bt = it.x, k = it.y;
        const int b = bt / p.tm.tiles, tile = bt % p.tm.tiles;
        const int axis = s.axis[b];
        const int thick = axis == 0 ? s.Z[0] : (axis == 1 ? s.Z[1] : s.Z[2]);
        scatter_body(p, tile, b, SlabCut{axis, k * thick, (k + 1) * thick});
    }
}

// Per-pose fixed-order sum of the item partials: thread j of the CTA takes
// tiles j, j + 256, ... in order and each tile's slabs in order.
__global__ void __launch_bounds__(256) slab_pose_reduce_kernel(const SlabParams s, int tiles, float* __restrict__ gM) {
    __shared__ float red[8][12];
    const int b = blockIdx.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float acc[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) acc[j] = 0.f;
    for (int t = tid; t < tiles; t += blockDim.x) {
        const int bt = b * tiles + t;
        const int n = s.count[bt];
        const float* pp = s.partials + (size_t)s.offset[bt] * kPartialStride;
        for (int q = 0; q < n; ++q) {
#pragma unroll
            for (int j = 0; j < 12; ++j) acc[j] += pp[(size_t)q * kPartialStride + j];
        }
    }
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        const float v = warp_sum(acc[j]);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (tid < 12) {
        float sum = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += red[w][tid];
        gM[(size_t)b * 12 + tid] = sum;
    }
}

template <typename VT, bool MULTI, int LAYOUT = kLayoutQuad>
static cudaError_t launch_slab_march(const MarchParams& p, const SlabParams& s, unsigned block, size_t smem,
                                     bool warp_agg, cudaStream_t st) {
    auto kern = warp_agg ? raymarch_bwd_slab_kernel<VT, MULTI, true, LAYOUT>
                         : raymarch_bwd_slab_kernel<VT, MULTI, false, LAYOUT>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)block, smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)std::max(1, sms * std::max(per_sm, 1));
    const KernelEvents& ev = kernel_events();
    if (ev.start != nullptr) cudaEventRecord(ev.start, st);
    kern<<<grid, block, smem, st>>>(p, s);
    e = cudaGetLastError();
    if (ev.stop != nullptr && e == cudaSuccess) e = cudaEventRecord(ev.stop, st);
    return e;
}

// Work list of a slab-ordered pass: the slab geometry and workspace carving
// in `s`, then the plan, scan and fill kernels on `st`.
static cudaError_t slab_setup(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p,
                              SlabParams& s, cudaStream_t st) {
    const SlabLayout L = slab_layout(a, ls);
    unsigned char* ws = reinterpret_cast<unsigned char*>(a.workspace);
    slab_geometry(a, s.Z, s.ns);
    s.base[0] = 0;
    s.base[1] = s.ns[0];
    s.base[2] = s.ns[0] + s.ns[1];
    s.ns_total = s.ns[0] + s.ns[1] + s.ns[2];
    s.BT = a.B * p.tm.tiles;
    s.counters = reinterpret_cast<int*>(ws + L.counters);
    s.hist = reinterpret_cast<int*>(ws + L.hist);
    s.key = reinterpret_cast<int*>(ws + L.key);
    s.trange = reinterpret_cast<int2*>(ws + L.trange);
    s.count = reinterpret_cast<int*>(ws + L.count);
    s.offset = reinterpret_cast<int*>(ws + L.offset);
    s.axis = reinterpret_cast<int*>(ws + L.axis);
    s.items = reinterpret_cast<int2*>(ws + L.items);
    s.partials = reinterpret_cast<float*>(ws + L.partials);
    cudaError_t e = cudaMemsetAsync(s.hist, 0, (size_t)s.ns_total * kSortBuckets * sizeof(int), st);
    if (e != cudaSuccess) return e;
    const int R = p.tw * p.th;
    slab_plan_kernel<<<s.BT, R, 0, st>>>(p, s);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    slab_scan_kernel<<<1, 1024, 0, st>>>(s);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    slab_fill_kernel<<<(s.BT + 255) / 256, 256, 0, st>>>(s, p.tm.tiles);
    return cudaGetLastError();
}

// The slab layout's partials region, which the split adjoint's pose pass
// uses for its per-tile partials (it holds at least one slot per tile).
float* slab_partials(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    return reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(a.workspace) + slab_layout(a, ls).partials);
}

// The split adjoint's scatter pass: slab-ordered, every sample of the cull
// window (no skip, no sample windows), into p.gquad (zeroed by the caller).
cudaError_t launch_scatter_slab(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p0,
                                cudaStream_t st) {
    MarchParams p = p0;
    p.win = nullptr;
    p.K = 1;
    SlabParams s;
    cudaError_t e = slab_setup(a, ls, p, s, st);
    if (e != cudaSuccess) return e;
    const int block = p.tw * p.th;
    int dev = 0, sms = 0, per_sm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, raymarch_scatter_slab_kernel, block, 0);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)std::max(1, sms * std::max(per_sm, 1));
    raymarch_scatter_slab_kernel<<<grid, block, 0, st>>>(p, s);
    return cudaGetLastError();
}

// Slab-ordered adjoint with volume gradient for the quad layout; writes gM
// and scatters into p.gquad (zeroed by the caller, folded afterwards).
cudaError_t launch_bwd_slab(const ndrr_raymarch_args& a, const LaunchShape& ls, const MarchParams& p0,
                            cudaStream_t st) {
    MarchParams p = p0;
    p.K = 1;  // items are short: one thread per ray
    // sample windows with a volume gradient gate the gathers only: every
    // sample of the cull window is scattered
    p.gwin = p0.win;
    p.win = nullptr;
    SlabParams s;
    cudaError_t e = slab_setup(a, ls, p, s, st);
    if (e != cudaSuccess) return e;
    p.partials = s.partials;
    const int R = p.tw * p.th;
    const size_t smem = bwd_epilogue_bytes(a, ls);
    const bool multi = a.n_classes > 1;
    const bool agg = a.gvol_mode == NDRR_GVOL_SLAB_WARP;
    const bool lab_quad = a.quad_labels != 0 && multi;  // validated: 16-bit volume with label channels
    switch (a.vol_dtype) {
        case NDRR_F32:
            e = multi ? launch_slab_march<float, true>(p, s, R, smem, agg, st)
                      : launch_slab_march<float, false>(p, s, R, smem, agg, st);
            break;
        case NDRR_F16:
            e = lab_quad ? launch_slab_march<__half, true, kLayoutQuadLab>(p, s, R, smem, agg, st)
                : multi  ? launch_slab_march<__half, true>(p, s, R, smem, agg, st)
                         : launch_slab_march<__half, false>(p, s, R, smem, agg, st);
            break;
        case NDRR_BF16:
            e = lab_quad ? launch_slab_march<__nv_bfloat16, true, kLayoutQuadLab>(p, s, R, smem, agg, st)
                : multi  ? launch_slab_march<__nv_bfloat16, true>(p, s, R, smem, agg, st)
                         : launch_slab_march<__nv_bfloat16, false>(p, s, R, smem, agg, st);
            break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    slab_pose_reduce_kernel<<<a.B, 256, 0, st>>>(s, p.tm.tiles, a.gM);
    return cudaGetLastError();
}

}  // namespace ndrr
