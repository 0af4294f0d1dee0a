// Measurement support, not part of the render path: the L2 read-bandwidth
// probe that gives the ray-march kernels' gather roofline its denominator,
// and the per-thread event hook that times a march kernel apart from the
// other launches of the same call (see ndrr_set_kernel_events).
#include "ndrr_march.cuh"

namespace ndrr {

thread_local KernelEvents g_kernel_events;

KernelEvents& kernel_events() { return g_kernel_events; }

// Every thread streams 16-byte words of `buf` `passes` times with
// ld.global.cg (cached in L2 only, so repeated passes are served by L2 and
// not by L1) and folds them into a register; the sink store happens only
// when the fold equals a value the caller's buffer never produces (zeros
// fold to 0), which keeps the loads alive without a store per thread.
__global__ void __launch_bounds__(512) l2_read_probe_kernel(const uint4* __restrict__ buf, unsigned long long n16,
                                                            int passes, unsigned* __restrict__ sink) {
    unsigned acc = 0u;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (int p = 0; p < passes; ++p) {
        for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n16; i += stride) {
            const uint4 v = __ldcg(buf + i);
            acc ^= (v.x ^ v.y) ^ (v.z ^ v.w);
        }
        acc = (acc << 1) | (acc >> 31);
    }
    if (acc == 0x9e3779b9u) atomicAdd(sink, 1u);
}

// Reduction-throughput probe: the volume-gradient scatter's access pattern
// alone. `buf` is read as planes of 512 x 512 16-byte quad entries; each warp
// is an 8 x 4 patch of rays one cell apart (x across lanes, planes down the
// patch) that steps 1 or 2 cells in y per sample and scatters each sample as
// two red.global.add.v4.f32 (its cell's entry in planes z and z + 1), with a
// per-warp pseudo-random origin. A buffer of a few tens of MiB stays in L2,
// so the probe measures the L2 reduction rate of that pattern. Indices: x <
// 504 + 8, y < 512, plane < planes - 4 + 3, plus one plane: inside `planes`.
constexpr int kProbeQX = 512;
constexpr long long kProbePlane = (long long)kProbeQX * kProbeQX;

__global__ void __launch_bounds__(512) reduce_probe_kernel(float4* __restrict__ buf, int planes, int iters) {
    const int lane = threadIdx.x & 31;
    const int lx = lane & 7, lz = lane >> 3;
    unsigned h = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 2654435761u + 12345u;
    int cy = (int)((h >> 7) % kProbeQX);
    for (int it = 0; it < iters; ++it) {
        h = h * 1664525u + 1013904223u;  // the same sequence in every lane of a warp
        cy = (cy + 1 + (int)((h >> 20) & 1u)) % kProbeQX;
        const int cx = (int)((h >> 8) % (unsigned)(kProbeQX - 8)) + lx;
        const int cz = (int)((h >> 24) % (unsigned)(planes - 4)) + lz;
        float* a = reinterpret_cast<float*>(buf + ((long long)cz * kProbeQX + cy) * kProbeQX + cx);
        float* b = a + kProbePlane * 4;
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(a), "f"(1.f), "f"(1.f), "f"(1.f),
                     "f"(1.f));
        asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(b), "f"(1.f), "f"(1.f), "f"(1.f),
                     "f"(1.f));
    }
}

cudaError_t launch_reduce_probe(void* buf, int planes, int iters, int sm_count, cudaStream_t st) {
    const unsigned grid = (unsigned)(sm_count > 0 ? sm_count * 4 : 4 * 148);
    reduce_probe_kernel<<<grid, 512, 0, st>>>(reinterpret_cast<float4*>(buf), planes, iters);
    return cudaGetLastError();
}

cudaError_t launch_l2_probe(const void* buf, unsigned long long bytes, int passes, unsigned* sink, int sm_count,
                            cudaStream_t st) {
    const unsigned long long n16 = bytes / 16;
    const unsigned grid = (unsigned)(sm_count > 0 ? sm_count * 4 : 4 * 148);
    l2_read_probe_kernel<<<grid, 512, 0, st>>>(reinterpret_cast<const uint4*>(buf), n16, passes, sink);
    return cudaGetLastError();
}

}  // namespace ndrr
