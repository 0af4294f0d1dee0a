// Persistent batched ray march: one launch renders many requests (volumes of
// one dtype, any detector size and sample count). Each CTA loops: it takes the
// next (request, tile) work item from an atomic counter, rebuilds the
// request's parameters from its descriptor and runs the same forward or
// adjoint tile body as the single-request kernels. Work items are numbered in
// request order; callers put the most expensive requests first so the tail
// of the launch is made of small tiles. No waits: a CTA exits when the
// counter passes the last item. A request with a quad-layout copy of its
// volume is marched from it (the choice is made per work item).
#include "ndrr_march.cuh"

namespace ndrr {

struct BatchParams {
    const ndrr_request* req;
    const int32_t* off;
    int n_req;
    int total;
    int lab_dtype, go_dtype, C;
    unsigned int* counter;
    float* partials;  // [total_tiles][kPartialStride]
};

__device__ __forceinline__ int find_request(const int32_t* __restrict__ off, int n, int item) {
    int lo = 0, hi = n;  // off[lo] <= item < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= item) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ MarchParams request_params(const BatchParams& bp, const ndrr_request& q, int r) {
    MarchParams p{};
    p.vol = q.vol;
    p.D = q.D;
    p.H = q.H;
    p.W = q.W;
    p.lab = q.lab;
    p.lab_dtype = bp.lab_dtype;
    p.C = bp.C;
    p.M = q.M;
    p.src = q.src;
    p.tgt = q.tgt;
    p.step = q.step;
    p.src_per_ray = q.src_per_ray;
    p.B = 1;
    p.N = q.N;
    p.S = q.n_samples;
    p.inv_s = 1.0f / (float)(q.n_samples - 1);
    p.out = q.out;
    p.go = q.go;
    p.go_dtype = bp.go_dtype;
    p.gsrc = q.gsrc;
    p.gtgt = q.gtgt;
    p.gstep = q.gstep;
    p.partials = bp.partials + (size_t)__ldg(bp.off + r) * kPartialStride;
    p.skip_mode = NDRR_SKIP_NONE;
    p.tw = q.tile_w;
    p.th = q.tile_h;
    p.K = q.sample_split;
    p.tm = make_tilemap(q.N, q.width, q.tile_w, q.tile_h);
    p.quad = q.vol_quad;
    p.qg = make_quadgeom(q.D, q.H, q.W);
    return p;
}

template <typename VT, bool MULTI>
__global__ void __launch_bounds__(256, 4) batched_fwd_kernel(const BatchParams bp) {
    __shared__ int s_item;
    for (;;) {
        __syncthreads();  // the previous item is done with s_item and smem
        if (threadIdx.x == 0) s_item = (int)atomicAdd(bp.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= bp.total) break;
        const int r = find_request(bp.off, bp.n_req, item);
        const MarchParams p = request_params(bp, bp.req[r], r);
        if (p.quad != nullptr)
            fwd_body<VT, VT, MULTI, 0, kLayoutQuad>(p, item - __ldg(bp.off + r), 0);
        else
            fwd_body<VT, VT, MULTI, 0, kLayoutVolume>(p, item - __ldg(bp.off + r), 0);
    }
}

template <typename VT, bool MULTI, bool GCAM>
__global__ void __launch_bounds__(256, 2) batched_bwd_kernel(const BatchParams bp) {
    __shared__ int s_item;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = (int)atomicAdd(bp.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= bp.total) break;
        const int r = find_request(bp.off, bp.n_req, item);
        const MarchParams p = request_params(bp, bp.req[r], r);
        const int tile = item - __ldg(bp.off + r);
        if (p.quad != nullptr)
            bwd_body<VT, MULTI, false, GCAM, 0, kLayoutQuad>(p, tile, 0, (size_t)tile);
        else
            bwd_body<VT, MULTI, false, GCAM, 0, kLayoutVolume>(p, tile, 0, (size_t)tile);
    }
}

// Per-request fixed-order sum of its tile partials (one CTA per request).
__global__ void __launch_bounds__(256) batched_reduce_kernel(const BatchParams bp, int gcam) {
    __shared__ float red[8][16];
    const int r = blockIdx.x;
    const ndrr_request& q = bp.req[r];
    const int t0 = __ldg(bp.off + r), t1 = __ldg(bp.off + r + 1);
    const bool shared_src = gcam && !q.src_per_ray;
    const int nterms = shared_src ? 15 : 12;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int j = 0; j < nterms; ++j) {
        float v = 0.f;
        for (int t = t0 + tid; t < t1; t += blockDim.x) v += bp.partials[(size_t)t * kPartialStride + j];
        v = warp_sum(v);
        if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (tid < nterms) {
        float sum = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += red[w][tid];
        if (tid < 12)
            q.gM[tid] = sum;
        else
            q.gsrc[tid - 12] = sum;
    }
}

static int default_ctas(int sm_count, int per_sm) { return sm_count * per_sm; }

template <typename VT>
static cudaError_t batched_fwd_dispatch(const BatchParams& bp, bool multi, int ctas, size_t smem, cudaStream_t st) {
    if (multi) {
        auto k = batched_fwd_kernel<VT, true>;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        k<<<ctas, 256, smem, st>>>(bp);
    } else {
        batched_fwd_kernel<VT, false><<<ctas, 256, smem, st>>>(bp);
    }
    return cudaGetLastError();
}

template <typename VT, bool MULTI>
static cudaError_t batched_bwd_dispatch2(const BatchParams& bp, bool gcam, int ctas, size_t smem, cudaStream_t st) {
    if (gcam)
        batched_bwd_kernel<VT, MULTI, true><<<ctas, 256, smem, st>>>(bp);
    else
        batched_bwd_kernel<VT, MULTI, false><<<ctas, 256, smem, st>>>(bp);
    return cudaGetLastError();
}

template <typename VT>
static cudaError_t batched_bwd_dispatch(const BatchParams& bp, bool multi, bool gcam, int ctas, size_t smem,
                                        cudaStream_t st) {
    return multi ? batched_bwd_dispatch2<VT, true>(bp, gcam, ctas, smem, st)
                 : batched_bwd_dispatch2<VT, false>(bp, gcam, ctas, smem, st);
}

static BatchParams make_batch(const ndrr_batch_args& a) {
    BatchParams bp;
    bp.req = a.requests;
    bp.off = a.tile_offsets;
    bp.n_req = a.n_requests;
    bp.total = a.total_tiles;
    bp.lab_dtype = a.lab_dtype;
    bp.go_dtype = a.go_dtype;
    bp.C = a.n_classes;
    bp.counter = reinterpret_cast<unsigned int*>(a.workspace);
    bp.partials = reinterpret_cast<float*>(reinterpret_cast<char*>(a.workspace) + 256);
    return bp;
}

cudaError_t launch_batched(const ndrr_batch_args& a, bool backward, int sm_count, cudaStream_t st) {
    const BatchParams bp = make_batch(a);
    cudaError_t e = cudaMemsetAsync(bp.counter, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    const bool multi = a.n_classes > 1, gcam = a.need_gcam != 0;
    if (!backward) {
        const int ctas = a.ctas > 0 ? a.ctas : default_ctas(sm_count, 4);
        const size_t smem = (multi ? (size_t)a.n_classes + 1 : 1) * 256 * sizeof(float);
        switch (a.vol_dtype) {
            case NDRR_F32: return batched_fwd_dispatch<float>(bp, multi, ctas, smem, st);
            case NDRR_F16: return batched_fwd_dispatch<__half>(bp, multi, ctas, smem, st);
            case NDRR_BF16: return batched_fwd_dispatch<__nv_bfloat16>(bp, multi, ctas, smem, st);
            default: return cudaErrorInvalidValue;
        }
    }
    const int ctas = a.ctas > 0 ? a.ctas : default_ctas(sm_count, 2);
    const size_t smem = std::max<size_t>((256 / 32) * kPartialStride, gcam ? 7 * 256 : 0) * sizeof(float);
    switch (a.vol_dtype) {
        case NDRR_F32: e = batched_bwd_dispatch<float>(bp, multi, gcam, ctas, smem, st); break;
        case NDRR_F16: e = batched_bwd_dispatch<__half>(bp, multi, gcam, ctas, smem, st); break;
        case NDRR_BF16: e = batched_bwd_dispatch<__nv_bfloat16>(bp, multi, gcam, ctas, smem, st); break;
        default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    batched_reduce_kernel<<<a.n_requests, 256, 0, st>>>(bp, gcam ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace ndrr
