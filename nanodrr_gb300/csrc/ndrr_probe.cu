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

cudaError_t launch_l2_probe(const void* buf, unsigned long long bytes, int passes, unsigned* sink, int sm_count,
                            cudaStream_t st) {
    const unsigned long long n16 = bytes / 16;
    const unsigned grid = (unsigned)(sm_count > 0 ? sm_count * 4 : 4 * 148);
    l2_read_probe_kernel<<<grid, 512, 0, st>>>(reinterpret_cast<const uint4*>(buf), n16, passes, sink);
    return cudaGetLastError();
}

}  // namespace ndrr
