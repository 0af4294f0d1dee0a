// TMA-staged forward: a measured variant of the ray march in which each CTA
// (a 16 x 8-ray detector tile) marches its rays in lockstep chunks of
// samples, and before a chunk is marched one thread copies the volume box
// that holds every corner the chunk's samples touch into shared memory with a
// 3-D TMA load (cp.async.bulk.tensor, completion on an mbarrier); the samples
// then gather their eight corners from shared memory. Two stages: the box of
// chunk c + 1 is in flight while chunk c is marched. The chunk length adapts
// so the box fits (32 x 16 x 16 voxels, 32 KB); a chunk whose box does not fit
// at one sample per chunk is marched from global memory instead. Out-of-volume
// voxels arrive as TMA zero fill, which is the renderer's zero padding, and
// the arithmetic is the software path's (same floor, fractions and lerps), so
// the image is bitwise that of the plain forward.
//
// Waits on the mbarriers are bounded. When a stage does not complete in
// time the CTA sets NDRR_FLAG_TMA_TIMEOUT in the library's device flags
// (read by ndrr_device_flags), waits again, bounded, for each of its copies
// still in flight so that none lands after the CTA's shared memory is
// released, writes NaN for its rays and returns.
#include <cuda.h>

#include "ndrr_march.cuh"

namespace ndrr {

// Box in voxels, x innermost. Measured at 512^3 x 32 poses x 256^2 x 800
// samples (ms): 32x32x16 6.94, 32x16x16 5.19, 32x32x8 11.7, 32x16x8 8.20,
// 32x8x8 8.49; the software quad path takes 2.18.
constexpr int kTBX = 32, kTBY = 16, kTBZ = 16;
constexpr int kTBoxElems = kTBX * kTBY * kTBZ;
constexpr unsigned kTBoxBytes = kTBoxElems * sizeof(float);  // 32 KB
constexpr int kTRays = 128;                                   // 16 x 8 tile, one thread per ray
constexpr int kTMaxChunk = 64;
constexpr int kTWaitLimit = 1 << 24;

// Library-wide device-side error flags (NDRR_FLAG_*), one word per device.
__device__ unsigned int g_ndrr_device_flags;

struct TmaShared {
    float box[2][kTBoxElems];
    unsigned long long bar[2];
    int origin[2][4];   // ox, oy, oz, valid
    int red[kTRays / 32][6];
    int chunk[2];       // sample range [c0, c1) of the next chunk
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(unsigned long long* b) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(b)) : "memory");
}

__device__ __forceinline__ void bar_expect(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool bar_try(unsigned long long* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool bar_wait(unsigned long long* b, unsigned parity) {
    for (int i = 0; i < kTWaitLimit; ++i)
        if (bar_try(b, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_box(float* dst, const CUtensorMap* map, int x, int y, int z,
                                             unsigned long long* b) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
          "r"(smem_u32(b))
        : "memory");
}

// Block-wide min of v[0..2] and max of v[3..5] (as min of negatives); the
// result lands in v for every thread.
__device__ __forceinline__ void block_box6(int (&v)[6], int (*red)[6]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        int x = v[k];
        for (int o = 16; o > 0; o >>= 1) x = min(x, __shfl_xor_sync(0xffffffffu, x, o));
        if (lane == 0) red[warp][k] = x;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        int x = red[0][k];
        for (int w = 1; w < kTRays / 32; ++w) x = min(x, red[w][k]);
        v[k] = x;
    }
    __syncthreads();
}

// Corner box of this ray's samples [a, e) (empty: neutral values).
__device__ __forceinline__ void ray_chunk_box(const ThreadRay& tr, const MarchParams& p, int a, int e, int (&v)[6]) {
    v[0] = v[1] = v[2] = INT_MAX;
    v[3] = v[4] = v[5] = INT_MAX;  // negated maxima
    if (a >= e) return;
    const float ta = (float)a * p.inv_s, te = (float)(e - 1) * p.inv_s;
    const float xa = floorf(fmaf(ta, tr.ray.dx, tr.ray.p0x)), xe = floorf(fmaf(te, tr.ray.dx, tr.ray.p0x));
    const float ya = floorf(fmaf(ta, tr.ray.dy, tr.ray.p0y)), ye = floorf(fmaf(te, tr.ray.dy, tr.ray.p0y));
    const float za = floorf(fmaf(ta, tr.ray.dz, tr.ray.p0z)), ze = floorf(fmaf(te, tr.ray.dz, tr.ray.p0z));
    v[0] = (int)fminf(xa, xe);
    v[1] = (int)fminf(ya, ye);
    v[2] = (int)fminf(za, ze);
    v[3] = -((int)fmaxf(xa, xe) + 1);  // the +1 corner
    v[4] = -((int)fmaxf(ya, ye) + 1);
    v[5] = -((int)fmaxf(za, ze) + 1);
}

__global__ void __launch_bounds__(kTRays) raymarch_fwd_tma_kernel(const MarchParams p,
                                                                       const __grid_constant__ CUtensorMap map) {
    extern __shared__ __align__(128) unsigned char tsm_raw[];
    TmaShared& sh = *reinterpret_cast<TmaShared*>(tsm_raw);
    const int tile = blockIdx.x % p.tm.tiles, b = blockIdx.x / p.tm.tiles;
    const int r = threadIdx.x;
    const int n = tile_ray(p.tm, p.N, p.tw, p.th, tile, r);
    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = __ldg(p.M + (size_t)b * 12 + j);
    ThreadRay tr;
    init_thread_ray(p, m, b, n, tr);
    const int lo = tr.ray.lo, hi = tr.ray.hi;

    if (threadIdx.x == 0) {
        bar_init(&sh.bar[0]);
        bar_init(&sh.bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // CTA sample range: union of the rays' windows
    int v[6] = {lo < hi ? lo : INT_MAX, 0, 0, lo < hi ? -hi : INT_MAX, 0, 0};
    block_box6(v, sh.red);
    const int s_begin = v[0], s_end = v[3] == INT_MAX ? 0 : -v[3];

    // Plans chunk [c0, c1) starting at c0 (length halved until its box fits
    // the stage), stores it, and (thread 0) issues its TMA load into `stage`.
    int len = 16;
    auto plan = [&](int c0, int stage) {
        int c1 = c0;
        bool fits = false;
        while (true) {
            c1 = min(s_end, c0 + len);
            int w[6];
            ray_chunk_box(tr, p, max(lo, c0), min(hi, c1), w);
            block_box6(w, sh.red);
            const int ox = w[0] == INT_MAX ? 0 : (w[0] & ~3);  // 16-byte aligned x start
            const int oy = w[1] == INT_MAX ? 0 : w[1], oz = w[2] == INT_MAX ? 0 : w[2];
            const bool empty = w[0] == INT_MAX;
            fits = empty || ((-w[3]) - ox < kTBX && (-w[4]) - oy < kTBY && (-w[5]) - oz < kTBZ);
            if (fits || len == 1) {
                if (threadIdx.x == 0) {
                    sh.chunk[stage] = c1;
                    sh.origin[stage][0] = ox;
                    sh.origin[stage][1] = oy;
                    sh.origin[stage][2] = oz;
                    sh.origin[stage][3] = fits && !empty ? 1 : 0;
                    if (fits && !empty) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        bar_expect(&sh.bar[stage], kTBoxBytes);
                        tma_load_box(sh.box[stage], &map, ox, oy, oz, &sh.bar[stage]);
                    }
                }
                break;
            }
            len = max(1, len >> 1);
        }
        if (fits && len < kTMaxChunk) len = min(kTMaxChunk, len * 2);
        __syncthreads();
    };

    float acc = 0.f;
    unsigned parity[2] = {0u, 0u};  // phase each stage's next completion ends
    bool failed = false;
    bool cur_pending = false;   // this thread's wait on the current stage gave up
    bool next_planned = false;  // a copy into the other stage was issued
    int c0 = s_begin;
    if (c0 < s_end) plan(c0, 0);
    int stage = 0;
    while (c0 < s_end) {
        const int c1 = sh.chunk[stage];
        const int ox = sh.origin[stage][0], oy = sh.origin[stage][1], oz = sh.origin[stage][2];
        const bool staged = sh.origin[stage][3] != 0;
        // stage the next chunk while this one is marched
        next_planned = c1 < s_end;
        if (next_planned) plan(c1, stage ^ 1);
        if (staged) {
            if (bar_wait(&sh.bar[stage], parity[stage])) {
                parity[stage] ^= 1u;
            } else {
                failed = true;
                cur_pending = true;
            }
        }
        const int a = max(lo, c0), e = min(hi, c1);
        if (!failed) {
            for (int s = a; s < e; ++s) {
                // the forward's float positions, so the image is bitwise its
                const float t = (float)s * p.inv_s;
                const float x = fmaf(t, tr.ray.dx, tr.ray.p0x);
                const float y = fmaf(t, tr.ray.dy, tr.ray.p0y);
                const float z = fmaf(t, tr.ray.dz, tr.ray.p0z);
                Cell c;
                if (staged) {
                    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
                    c.fx = x - xf;
                    c.fy = y - yf;
                    c.fz = z - zf;
                    const int lx = (int)xf - ox, ly = (int)yf - oy, lz = (int)zf - oz;
                    const float* bx = sh.box[stage] + (lz * kTBY + ly) * kTBX + lx;
                    c.v000 = bx[0];
                    c.v001 = bx[1];
                    c.v010 = bx[kTBX];
                    c.v011 = bx[kTBX + 1];
                    c.v100 = bx[kTBX * kTBY];
                    c.v101 = bx[kTBX * kTBY + 1];
                    c.v110 = bx[kTBX * kTBY + kTBX];
                    c.v111 = bx[kTBX * kTBY + kTBX + 1];
                } else {
                    load_cell(reinterpret_cast<const float*>(p.vol), p.D, p.H, p.W, x, y, z, c);
                }
                acc += cell_value(c);
            }
        }
        // every thread is done with this stage before it is refilled, and a
        // timed-out wait anywhere stops the whole CTA
        failed = __syncthreads_or(failed) != 0;
        if (failed) break;
        c0 = c1;
        stage ^= 1;
    }
    if (failed) {
        // A stage did not complete in time: flag it for the host, then wait
        // again (bounded) for the copies this thread has not seen complete —
        // the current stage if its own wait gave up, and the other stage if
        // a copy was issued into it — before the CTA exits; its rays read NaN.
        if (threadIdx.x == 0) atomicOr(&g_ndrr_device_flags, (unsigned)NDRR_FLAG_TMA_TIMEOUT);
        if (cur_pending) bar_wait(&sh.bar[stage], parity[stage]);
        const int other = stage ^ 1;
        if (next_planned && sh.origin[other][3] != 0) bar_wait(&sh.bar[other], parity[other]);
        acc = __int_as_float(0x7fc00000);
    }
    if (n >= 0) st_out(reinterpret_cast<float*>(p.out), tr.bn, acc * tr.stepv);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The CUDA driver's tensor-map encoder, looked up once (thread-safe static init).
static EncodeTiledFn encode_fn() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(f);
        return nullptr;
    }();
    return fn;
}

size_t tma_fwd_smem_bytes() { return sizeof(TmaShared) + 128; }

cudaError_t launch_fwd_tma(const ndrr_raymarch_args& a, const LaunchShape& ls, cudaStream_t st) {
    EncodeTiledFn enc = encode_fn();
    if (enc == nullptr) return cudaErrorNotSupported;
    CUtensorMap map;
    const cuuint64_t dims[3] = {(cuuint64_t)a.W, (cuuint64_t)a.H, (cuuint64_t)a.D};
    const cuuint64_t strides[2] = {(cuuint64_t)a.W * sizeof(float), (cuuint64_t)a.W * a.H * sizeof(float)};
    const cuuint32_t box[3] = {kTBX, kTBY, kTBZ};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult cr = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(a.vol), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return cudaErrorInvalidValue;
    LaunchShape ts = ls;  // the kernel is built for 16 x 8 tiles, one thread per ray
    ts.tw = 16;
    ts.th = 8;
    ts.K = 1;
    MarchParams p = make_params(a, ts);
    const size_t smem = tma_fwd_smem_bytes();
    cudaError_t e = cudaFuncSetAttribute(raymarch_fwd_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)((size_t)a.B * p.tm.tiles);
    raymarch_fwd_tma_kernel<<<grid, kTRays, smem, st>>>(p, map);
    return cudaGetLastError();
}

// Read (and optionally clear) the device flags of the current device.
// Synchronous: the copy waits for the device's work to finish.
cudaError_t device_flags(unsigned* out, bool clear) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_ndrr_device_flags, sizeof(unsigned));
    if (e == cudaSuccess && clear) {
        const unsigned zero = 0u;
        e = cudaMemcpyToSymbol(g_ndrr_device_flags, &zero, sizeof(unsigned));
    }
    return e;
}

}  // namespace ndrr
