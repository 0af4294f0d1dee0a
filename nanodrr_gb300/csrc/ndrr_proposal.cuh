// Learned empty-space proposal: a 3-layer MLP that maps a ray to the part of
// its in-volume segment that is not air.
//
// Input: the ray's entry and exit points of the footprint box (-1, dim) in
// volume-normalised coordinates (voxel / dim), Fourier-encoded:
//   f = [v, sin(pi 2^k v), cos(pi 2^k v) for k = 0..3]  (6 + 48 = 54, zero-padded to 64).
// Network: 64 -> 64 (ReLU) -> 64 (ReLU) -> 2, predicting the fractions
// (f_near, f_far) of the in-box segment [tau0, tau1] where the non-empty
// interval starts and ends; t_near = tau0 + f_near (tau1 - tau0).
//
// Inference runs in the window kernel (ndrr_windows.cu), together with the
// occupancy check, on the tensor cores with warp-level mma.sync (bf16
// operands, fp32 accumulation): a warp evaluates its 32 rays as two 16-row
// tiles, keeping layer outputs in registers (an m16n8 f32 accumulator pair is
// exactly the A operand of the next m16n8k16 step).
#pragma once

#include "ndrr_device.cuh"

namespace ndrr {

constexpr int kPropIn = 64;
constexpr int kPropHidden = 64;
constexpr int kPropOut = 2;
constexpr int kPropFeatures = 54;  // used inputs; the rest are zero

// fp32 master parameter layout (training): W1 [64][64], b1 [64], W2 [64][64],
// b2 [64], W3 [2][64], b3 [2]; weights row-major [out][in].
constexpr int kPropW1 = 0;
constexpr int kPropB1 = kPropW1 + kPropHidden * kPropIn;
constexpr int kPropW2 = kPropB1 + kPropHidden;
constexpr int kPropB2 = kPropW2 + kPropHidden * kPropHidden;
constexpr int kPropW3 = kPropB2 + kPropHidden;
constexpr int kPropB3 = kPropW3 + kPropOut * kPropHidden;
constexpr int kPropParams = kPropB3 + kPropOut;  // 8450 floats

// Packed inference layout (bytes): bf16 W1 [64][64], W2 [64][64], W3 [8][64]
// (rows 2..7 zero), then f32 b1 [64], b2 [64], b3 [8].
constexpr int kPackW1 = 0;
constexpr int kPackW2 = kPackW1 + 64 * 64 * 2;
constexpr int kPackW3 = kPackW2 + 64 * 64 * 2;
constexpr int kPackB1 = kPackW3 + 8 * 64 * 2;
constexpr int kPackB2 = kPackB1 + 64 * 4;
constexpr int kPackB3 = kPackB2 + 64 * 4;
constexpr int kPackBytes = kPackB3 + 8 * 4;  // 17952

// Shared-memory layout of the inference: weight rows padded to 72 bf16
// (144 B: the 8 rows x 4 column pairs a fragment load touches fall in 32
// distinct banks), per-warp feature staging [32][72] bf16, per-ray results.
constexpr int kRowPad = 72;
constexpr int kSmW1 = 0;
constexpr int kSmW2 = kSmW1 + 64 * kRowPad * 2;
constexpr int kSmW3 = kSmW2 + 64 * kRowPad * 2;
constexpr int kSmBias = kSmW3 + 8 * kRowPad * 2;          // f32 b1[64] b2[64] b3[8]
constexpr int kSmStage = kSmBias + (64 + 64 + 8) * 4;     // per-warp [32][72] bf16
constexpr int kSmStageWarp = 32 * kRowPad * 2;

__host__ __device__ constexpr size_t proposal_smem_bytes(int rays_per_cta) {
    return (size_t)kSmStage + (size_t)(rays_per_cta / 32) * kSmStageWarp + (size_t)rays_per_cta * 8;
}

// In-box segment [tau0, tau1] of the ray's line and the 64 input features.
// Returns false when the line misses the footprint box.
__device__ __forceinline__ bool proposal_features(const Ray& r, int D, int H, int W, float& tau0, float& tau1,
                                                  float (&f)[kPropIn]) {
    float ax0, ax1, ay0, ay1, az0, az1;
    axis_interval(r.p0x, r.dx, -1.0f, (float)W, ax0, ax1);
    axis_interval(r.p0y, r.dy, -1.0f, (float)H, ay0, ay1);
    axis_interval(r.p0z, r.dz, -1.0f, (float)D, az0, az1);
    tau0 = fmaxf(fmaxf(ax0, ay0), az0);
    tau1 = fminf(fminf(ax1, ay1), az1);
    const bool hit = tau0 < tau1 && isfinite(tau0) && isfinite(tau1);
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (hit) {
        v[0] = fmaf(tau0, r.dx, r.p0x) / (float)W;
        v[1] = fmaf(tau0, r.dy, r.p0y) / (float)H;
        v[2] = fmaf(tau0, r.dz, r.p0z) / (float)D;
        v[3] = fmaf(tau1, r.dx, r.p0x) / (float)W;
        v[4] = fmaf(tau1, r.dy, r.p0y) / (float)H;
        v[5] = fmaf(tau1, r.dz, r.p0z) / (float)D;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        f[i] = v[i];
        // sin/cos of pi v, then the double-angle recurrences for 2x, 4x, 8x.
        float s, c;
        sincospif(v[i], &s, &c);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            f[6 + k * 12 + i] = s;
            f[6 + k * 12 + 6 + i] = c;
            const float s2 = 2.f * s * c, c2 = 1.f - 2.f * s * s;
            s = s2;
            c = c2;
        }
    }
#pragma unroll
    for (int i = kPropFeatures; i < kPropIn; ++i) f[i] = 0.f;
    return hit;
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t lds32(const unsigned char* base, int byte_off) {
    return *reinterpret_cast<const uint32_t*>(base + byte_off);
}

// Copy the packed parameters into the padded shared-memory layout. All threads
// of the CTA call this; the caller synchronises afterwards.
__device__ __forceinline__ void proposal_stage_weights(const unsigned char* __restrict__ packed, unsigned char* sm) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(packed);
    // weights: 64 + 64 + 8 rows of 32 words each
    for (int i = threadIdx.x; i < (64 + 64 + 8) * 32; i += blockDim.x) {
        const int row = i >> 5, w = i & 31;
        *reinterpret_cast<uint32_t*>(sm + row * kRowPad * 2 + w * 4) = __ldg(src + row * 32 + w);
    }
    const float* bias = reinterpret_cast<const float*>(packed + kPackB1);
    for (int i = threadIdx.x; i < 64 + 64 + 8; i += blockDim.x)
        reinterpret_cast<float*>(sm + kSmBias)[i] = __ldg(bias + i);
}

// One hidden layer for one 16-ray tile: out = relu(W x + b), consuming and
// producing A-operand fragments [kchunk][4].
__device__ __forceinline__ void proposal_hidden_layer(const unsigned char* sm_w, const float* sm_b,
                                                      const uint32_t (&ain)[4][4], uint32_t (&aout)[4][4], int g,
                                                      int tig) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // output k-chunk q = n-tiles 2q, 2q + 1
        float acc[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = 2 * q + h;
            const float b0 = sm_b[8 * j + 2 * tig], b1 = sm_b[8 * j + 2 * tig + 1];
            acc[h][0] = b0;
            acc[h][1] = b1;
            acc[h][2] = b0;
            acc[h][3] = b1;
#pragma unroll
            for (int kc = 0; kc < 4; ++kc) {
                const int row = 8 * j + g;
                const uint32_t w0 = lds32(sm_w, (row * kRowPad + 16 * kc + 2 * tig) * 2);
                const uint32_t w1 = lds32(sm_w, (row * kRowPad + 16 * kc + 8 + 2 * tig) * 2);
                mma_bf16_16816(acc[h], ain[kc], w0, w1);
            }
        }
        aout[q][0] = pack_bf16x2(fmaxf(acc[0][0], 0.f), fmaxf(acc[0][1], 0.f));
        aout[q][1] = pack_bf16x2(fmaxf(acc[0][2], 0.f), fmaxf(acc[0][3], 0.f));
        aout[q][2] = pack_bf16x2(fmaxf(acc[1][0], 0.f), fmaxf(acc[1][1], 0.f));
        aout[q][3] = pack_bf16x2(fmaxf(acc[1][2], 0.f), fmaxf(acc[1][3], 0.f));
    }
}

// Proposed [pn, pf] (in t) for every ray of the CTA's current item. Called by
// all threads after proposal_stage_weights (done once per persistent CTA);
// rays are CTA-local indices r in [0, R) owned by the threads with k == 0
// (warps never mix k). `sm` is the proposal shared-memory region.
__device__ __forceinline__ void proposal_window_cta(unsigned char* sm, const Ray& ray, int D, int H, int W,
                                                    bool has, int r, int k, int R, float& pn, float& pf) {
    __syncthreads();  // the previous tile is done with the result slots
    float* res = reinterpret_cast<float*>(sm + kSmStage + (R / 32) * kSmStageWarp);  // [R][2]
    const int lane = threadIdx.x & 31;
    if (k == 0) {
        const int warp = r >> 5;
        unsigned char* stage = sm + kSmStage + warp * kSmStageWarp;
        float tau0 = 0.f, tau1 = 0.f;
        float f[kPropIn];
        const bool hit = proposal_features(ray, D, H, W, tau0, tau1, f) && has;
        // Stage this lane's ray as row `lane` (bf16).
#pragma unroll
        for (int i = 0; i < kPropIn; i += 2)
            *reinterpret_cast<uint32_t*>(stage + (lane * kRowPad + i) * 2) = pack_bf16x2(f[i], f[i + 1]);
        __syncwarp();
        const int g = lane >> 2, tig = lane & 3;
        const float* bias = reinterpret_cast<const float*>(sm + kSmBias);
        float* wres = res + warp * 64;
        // The warp's 32 rays are two 16-row tiles; both are unrolled so their
        // mma chains interleave (the window kernel has registers to spare:
        // 0.53 ms instead of 0.59 ms for 2.1 M rays).
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            uint32_t a0[4][4], a1[4][4];
            const int r0 = mt * 16 + g, r1 = r0 + 8;
#pragma unroll
            for (int kc = 0; kc < 4; ++kc) {
                a0[kc][0] = lds32(stage, (r0 * kRowPad + 16 * kc + 2 * tig) * 2);
                a0[kc][1] = lds32(stage, (r1 * kRowPad + 16 * kc + 2 * tig) * 2);
                a0[kc][2] = lds32(stage, (r0 * kRowPad + 16 * kc + 8 + 2 * tig) * 2);
                a0[kc][3] = lds32(stage, (r1 * kRowPad + 16 * kc + 8 + 2 * tig) * 2);
            }
            proposal_hidden_layer(sm + kSmW1, bias, a0, a1, g, tig);
            proposal_hidden_layer(sm + kSmW2, bias + 64, a1, a0, g, tig);
            // Output layer: one n-tile (rows 0, 1 of W3 are used).
            float out[4];
            const float b0 = bias[128 + 2 * tig], b1 = bias[128 + 2 * tig + 1];
            out[0] = b0;
            out[1] = b1;
            out[2] = b0;
            out[3] = b1;
#pragma unroll
            for (int kc = 0; kc < 4; ++kc) {
                const uint32_t w0 = lds32(sm + kSmW3, (g * kRowPad + 16 * kc + 2 * tig) * 2);
                const uint32_t w1 = lds32(sm + kSmW3, (g * kRowPad + 16 * kc + 8 + 2 * tig) * 2);
                mma_bf16_16816(out, a0[kc], w0, w1);
            }
            // Columns 0, 1 live in the tig == 0 lanes: rows g and g + 8.
            if (tig == 0) {
                wres[r0 * 2 + 0] = out[0];
                wres[r0 * 2 + 1] = out[1];
                wres[r1 * 2 + 0] = out[2];
                wres[r1 * 2 + 1] = out[3];
            }
        }
        __syncwarp();
        const float fn = wres[lane * 2 + 0], ff = wres[lane * 2 + 1];
        const float span = tau1 - tau0;
        // Rays that miss the box, or have no window: an empty proposal.
        wres[lane * 2 + 0] = hit ? fmaf(fn, span, tau0) : 1.f;
        wres[lane * 2 + 1] = hit ? fmaf(ff, span, tau0) : 0.f;
    }
    __syncthreads();
    pn = res[r * 2 + 0];
    pf = res[r * 2 + 1];
}

}  // namespace ndrr
