/*
 * nanodrr_gb300 — C ABI of the GB300 (sm_103a) differentiable ray-march renderer.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream handle
 * (a `cudaStream_t` passed as `void*`; NULL is the legacy default stream). No
 * entry point allocates device memory, synchronises the stream or calls into a
 * framework: scratch memory is passed in by the caller, sized by the matching
 * `*_workspace_bytes` query. All launches are asynchronous on `stream`.
 *
 * Return value: NDRR_OK (0) or one of the NDRR_ERR_* codes below; the message
 * of the last failure on the calling thread is returned by ndrr_last_error().
 *
 * Alignment: every device pointer must be aligned to its element size, and
 * the arrays the kernels move 16 bytes at a time to 16 bytes: vol_quad,
 * gvol_quad, the workspace, and gvol when the quad layout is used (the
 * quad-gradient fold writes four floats per store). Misaligned pointers are
 * refused with NDRR_ERR_INVALID_ARGUMENT before anything is launched.
 * Allocations from cudaMalloc and from the torch caching allocator always
 * qualify; offset views into a pooled buffer may not.
 *
 * Coordinate conventions (identical to the reference renderer):
 *   - the volume is a dense row-major [D, H, W] array; voxel (x, y, z) is
 *     element (z * H + y) * W + x;
 *   - sample positions are computed from the inputs in float-float and
 *     carried in 32.32 fixed point, not rounded to float32 (see M_lo);
 *   - M is a per-pose 3x4 row-major affine from camera space (mm) to voxel
 *     index space, so sample s of ray n sits at
 *         p = M @ [lerp(src_n, tgt_n, t_s), 1],  t_s = s / (n_samples - 1);
 *   - each sample is a trilinear interpolation with zero padding per corner
 *     (grid_sample bilinear, align_corners=False in voxel-index form);
 *   - with n_classes > 1 each sample is routed to the channel given by the
 *     nearest label (round half to even) at the same position; labels outside
 *     [0, n_classes) are dropped;
 *   - out[b, c, n] = step[b, n] * sum of the samples routed to channel c.
 */
#ifndef NANODRR_GB300_H
#define NANODRR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NDRR_ABI_VERSION 3

#if defined(__GNUC__)
#define NDRR_API __attribute__((visibility("default")))
#else
#define NDRR_API
#endif

/* ---- status codes --------------------------------------------------------- */
enum ndrr_status {
    NDRR_OK = 0,
    NDRR_ERR_INVALID_ARGUMENT = 1, /* bad shape, null pointer, n_samples < 2 ...  */
    NDRR_ERR_LIMIT = 2,            /* exceeds the int32 indexing or channel limits */
    NDRR_ERR_DTYPE = 3,            /* unsupported element type                     */
    NDRR_ERR_WORKSPACE = 4,        /* workspace missing or too small               */
    NDRR_ERR_CUDA = 5,             /* a CUDA runtime call or launch failed         */
    NDRR_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up           */
};

/* ---- element types -------------------------------------------------------- */
enum ndrr_dtype {
    NDRR_F32 = 0,
    NDRR_F16 = 1,
    NDRR_BF16 = 2,
    NDRR_U8 = 3,
    NDRR_I8 = 4,
    NDRR_I16 = 5,
    NDRR_I32 = 6,
    NDRR_I64 = 7,
};

/* ---- ray-march arguments --------------------------------------------------- *
 * One struct serves the forward and the adjoint; fields a call does not use
 * may be zero/NULL. Pointers are device pointers unless stated otherwise.     */
typedef struct ndrr_raymarch_args {
    uint32_t struct_size;   /* sizeof(ndrr_raymarch_args), checked by the library */
    uint32_t abi_version;   /* NDRR_ABI_VERSION                                   */

    /* Volume [D, H, W], contiguous: f32, f16 or bf16. */
    const void* vol;
    int32_t vol_dtype;
    int32_t D, H, W;

    /* Label map [D, H, W], contiguous, any ndrr_dtype; read only when
     * n_classes > 1. Float labels are truncated toward zero like a cast. */
    const void* lab;
    int32_t lab_dtype;
    int32_t n_classes;      /* C >= 1 */

    /* Geometry. M: [B, 3, 4] f32. src: [B, 1, 3] (src_per_ray = 0, one source
     * per pose) or [B, N, 3] (src_per_ray = 1), f32. tgt: [B, N, 3] f32.
     * step: [B, N] f32 (camera-space sample spacing, mm). All contiguous. */
    const float* M;
    const float* src;
    const float* tgt;
    const float* step;
    int32_t src_per_ray;
    int32_t B;              /* poses                                            */
    int32_t N;              /* rays per pose                                    */
    int32_t width;          /* detector width; rays form a (N / width) x width
                               image when width > 0 and divides N, else a list */
    int32_t n_samples;      /* samples per ray, >= 2                            */

    /* Optional per-ray sample window [B, N, 2] f32 in units of t (0 = src,
     * 1 = tgt), or NULL. Samples with t outside [lo, hi] are skipped. Used by
     * the empty-space proposal; NULL marches the full (box-culled) ray. */
    const float* t_window;

    /* Forward output [B, C, N], dtype out_dtype (f32, f16 or bf16). When
     * out_total is non-NULL it receives the unrouted line integral [B, N]
     * (the single-channel render) in out_dtype as well. */
    void* out;
    int32_t out_dtype;
    void* out_total;

    /* Adjoint inputs/outputs. go: [B, C, N] upstream gradient, dtype go_dtype.
     * gvol: [D, H, W] f32, ACCUMULATED into (zero it first).
     * gM: [B, 3, 4] f32, written. gsrc: [B, 1, 3] or [B, N, 3] f32 (following
     * src_per_ray), gtgt: [B, N, 3] f32 and gstep: [B, N] f32, written when
     * need_gcam. */
    const void* go;
    int32_t go_dtype;
    int32_t need_gvol;
    int32_t need_gcam;
    float* gvol;
    float* gM;
    float* gsrc;
    float* gtgt;
    float* gstep;

    /* Scratch for the adjoint's deterministic per-tile pose partials. */
    void* workspace;
    uint64_t workspace_bytes;

    /* Empty-space skipping (optional; see ndrr_occupancy_build).
     * skip_mode NDRR_SKIP_OCCUPANCY: each ray marches only between the first
     * and last occupied grid cell it crosses (computed inside the render
     * kernels, or ahead of them by ndrr_skip_windows). NDRR_SKIP_PROPOSAL:
     * the learned proposal network (proposal_params, packed by
     * ndrr_proposal_pack) predicts the non-empty interval; the occupancy grid
     * then checks that nothing occupied lies outside it, and rays that fail
     * the check march their full box-culled window. The proposal is computed
     * by ndrr_skip_windows only; the march entry points reject skip_mode 2
     * (pass the windows as sample_window). Skipped samples have eight zero
     * corners, so the image and the pose and camera gradients are unchanged;
     * the volume gradient, which is non-zero on empty voxels too, always uses
     * the full window (the adjoint ignores the skip when need_gvol is set). */
    int32_t skip_mode;
    int32_t occ_cell;
    int32_t occ_gx, occ_gy, occ_gz;
    const uint8_t* occ_grid;
    const void* proposal_params;
    float proposal_margin;          /* widening of a proposed interval, samples */
    unsigned long long* skip_stats; /* optional [4] counters, accumulated: rays
                                       with a window, rays sent to the full
                                       march, samples marched, samples in the
                                       box-culled windows */
    float* out_extent;              /* optional [B, N, 2] forward output: t of
                                       the first and last sample with a
                                       non-zero corner, (1, 0) when none */

    /* Quad layout (optional, built by ndrr_quad_build from `vol`): when
     * vol_quad is set the kernels read each sample's eight corners with two
     * vector loads from it instead of eight gathers from vol (same values,
     * same results). The adjoint with need_gvol then also needs gvol_quad, a
     * float32 scratch of ndrr_quad_dims elements x 16 bytes, which it zeroes,
     * scatters into with two 16-byte reductions per sample and folds into
     * gvol. Forward output in the volume's dtype only. */
    const void* vol_quad;
    float* gvol_quad;

    /* Optional per-ray sample windows [B, N, 2] int32 (first sample, one
     * past the last), as written by ndrr_skip_windows, or NULL. Each ray
     * marches only the samples of its window (intersected with its box-culled
     * window). It is an empty-space window (samples outside it have eight
     * zero corners): valid for the forward and the pose/camera adjoint, and
     * with need_gvol for the slab-ordered adjoint of one channel (gvol_mode
     * 0, 3, 4 with the quad layout), where it only spares the loads of the
     * samples outside (every sample is still scattered into the volume
     * gradient; results unchanged), and for gvol_mode 5 (its pose pass).
     * Rejected with the other need_gvol paths and with skip_mode (one skip
     * at a time). */
    const int32_t* sample_window;

    /* Launch tuning; 0 selects the library default for each. */
    int32_t tile_w;         /* detector tile width in rays (8 or 16)            */
    int32_t tile_h;         /* detector tile height in rays (8 or 16)           */
    int32_t sample_split;   /* 1, 2, 4, 8 or 16 sample chunks per ray within a
                               CTA (tile_w * tile_h * sample_split <= 512)      */
    int32_t gvol_mode;      /* adjoint volume-gradient scatter: 0 auto,
                               1 direct global atomics per tap, 2 per-slab
                               shared-memory brick flushed with coalesced
                               atomics, 3 slab-ordered work (quad layout, no
                               camera gradients; see NDRR_GVOL_SLAB), 4 slab
                               with warp aggregation, 5 split pose and scatter
                               passes (NDRR_GVOL_*)                             */
    int32_t brick_cap;      /* gvol_mode 2: brick capacity in voxels (0 default,
                               at most 57344)                                   */
    int32_t slab_mib;       /* gvol_mode 3 (and auto): quad-gradient MiB per
                               slab (0 default = 128, at most 4096)              */
    int32_t fwd_mode;       /* NDRR_FWD_* (0 default)                          */
    int32_t gvol_overwrite; /* quad layout only: 1 = the adjoint writes gvol
                               instead of accumulating into it (no zeroing
                               needed); rejected without vol_quad              */
    /* Texture-filtered forward (a measured variant, not the default): a
     * handle from ndrr_texture_create. When set, ndrr_raymarch_fwd samples
     * it with the texture unit's trilinear filter, whose interpolation
     * weights have 8 fractional bits (results differ from the fp32 path by
     * about 1e-3 relative); one channel, no skipping, no quad layout. */
    uint64_t vol_texture;

    /* Labelled quad layout (16-bit volumes with n_classes in 2..255): set to
     * 1 when vol_quad was built by ndrr_quad_build_labeled. Each 16-byte
     * element then also carries its four corners' classes, so a per-label
     * sample takes its nearest label from the two loads that bring its
     * corners instead of a third gather from `lab` (same routing, same
     * results). lab stays required and is what the other paths read. */
    int32_t quad_labels;
    int32_t reserved0;

    /* Optional low parts of M, [B, 3, 4] f32, or NULL: the affine is taken as
     * M + M_lo (a float64 affine split into two floats, ~2^-48 relative).
     * Sample positions are formed from it in float-float and carried in 32.32
     * fixed point (about 2e-7 voxel after 800 samples), so a sample falls in
     * the cell the exact position falls in; with M_lo NULL the float32 M is
     * taken as exact. */
    const float* M_lo;
} ndrr_raymarch_args;

/* Forward variants (ndrr_raymarch_args.fwd_mode). */
enum ndrr_fwd_mode {
    NDRR_FWD_DEFAULT = 0,  /* software trilinear from the volume or quad layout */
    NDRR_FWD_TMA = 1,      /* measured variant: per-tile volume boxes staged into
                              shared memory by 3-D TMA loads (f32 volume with W a
                              multiple of 4, one channel, f32 output, no skipping,
                              windows or quad layout); bitwise the default's
                              image */
};

enum ndrr_skip_mode {
    NDRR_SKIP_NONE = 0,
    NDRR_SKIP_OCCUPANCY = 1,
    NDRR_SKIP_PROPOSAL = 2,
};

/* NDRR_GVOL_SLAB: the volume is cut into slabs (about 128 MB of quad
 * gradient each) along one axis per pose, and (slab, pose, tile) work items
 * run slab by slab across all poses, so that a slab's lines are reused from
 * L2 by every pose before eviction. It is what NDRR_GVOL_AUTO selects for
 * the quad layout without camera gradients. Needs a larger workspace (work
 * list and per-item pose partials: ndrr_raymarch_bwd_workspace_bytes
 * reports it); gM stays deterministic (fixed partial slots and summation
 * order). */
enum ndrr_gvol_mode {
    NDRR_GVOL_AUTO = 0,
    NDRR_GVOL_DIRECT = 1,
    NDRR_GVOL_BRICK = 2,
    NDRR_GVOL_SLAB = 3,
    NDRR_GVOL_SLAB_WARP = 4, /* NDRR_GVOL_SLAB with warp aggregation: lanes of a
                                warp scattering into the same quad cell in the
                                same step combine their terms before the
                                reduction (__match_any_sync + shuffles)      */
    NDRR_GVOL_SPLIT = 5,     /* two passes: the pose adjoint (the volume
                                gathers; honours sample_window and
                                skip_mode, whose skipped samples carry no pose
                                terms), then the volume-gradient scatter in
                                slab order from sample positions alone (no
                                gathers). Quad layout, one channel, no camera
                                gradients (else NDRR_GVOL_SLAB); the workspace
                                is NDRR_GVOL_SLAB's. Measured slower than
                                NDRR_GVOL_SLAB (8.65 against 6.79 ms at 512^3,
                                32 x 256^2): the scatter is the bound      */
};

/* Library identity. */
NDRR_API int32_t ndrr_abi_version(void);
NDRR_API const char* ndrr_build_info(void);

/* Message of the last failed call on this thread ("" if none). */
NDRR_API const char* ndrr_last_error(void);

/* Device-side error flags of this library on the current device, set by
 * kernels that cannot return a status through a launch:
 * NDRR_FLAG_TMA_TIMEOUT — a TMA-staged forward (NDRR_FWD_TMA) gave up waiting
 * for a shared-memory stage; the rays of that tile were written as NaN.
 * *flags receives the word; clear = 1 resets it. Unlike every other entry
 * point this one synchronises: the read waits for the device's work. */
#define NDRR_FLAG_TMA_TIMEOUT 1u
NDRR_API int32_t ndrr_device_flags(uint32_t* flags, int32_t clear);

/* Forward ray march. Replaces the custom op nanodrr::fused_raymarch
 * (reference src/nanodrr/drr/_fused.py:415-460): same inputs (vol, lab, M,
 * src, tgt, step, n_samples, n_classes, width), caller-allocated output. The
 * split-partials buffer and the final sum/cast of the reference are not
 * needed: the output is reduced inside each CTA and written in out_dtype. */
NDRR_API int32_t ndrr_raymarch_fwd(const ndrr_raymarch_args* args, void* stream);

/* Bytes of scratch ndrr_raymarch_bwd needs for `args` (0 is possible). */
NDRR_API int32_t ndrr_raymarch_bwd_workspace_bytes(const ndrr_raymarch_args* args, uint64_t* bytes);

/* Adjoint ray march. Replaces nanodrr::fused_raymarch_bwd (reference
 * src/nanodrr/drr/_fused.py:477-531): recomputes the samples, writes the pose
 * gradient gM deterministically (fixed-order reduction of per-tile partials),
 * optional camera-space gradients (gsrc summed over rays when src is one per
 * pose, as the reference's _backward does at _fused.py:552-553) and
 * accumulates the volume gradient with atomics (not bitwise deterministic). */
NDRR_API int32_t ndrr_raymarch_bwd(const ndrr_raymarch_args* args, void* stream);

/* Allocation-free adjoint: the same computation and arguments as
 * ndrr_raymarch_bwd, but args->workspace is ignored and the per-tile pose
 * partials go to a 4 MiB scratch array inside this library, so the call needs
 * no device allocation at all. It is meant for callers that cannot allocate
 * device memory where they run the adjoint: hosts that own every byte of
 * device memory through their own pool and give plugins no allocator, and
 * real-time loops in which a cudaMalloc (with its implicit synchronisation
 * and unbounded latency) is not allowed. Limits and behaviour:
 *   - at most 4 MiB of partials (16 floats per pose and detector tile, e.g.
 *     65536 pose-tiles = 128 poses of 256 x 256 rays with 16 x 8 tiles);
 *     larger calls fail with NDRR_ERR_LIMIT and a message;
 *   - the array is held by every GPU that loads the library until exit;
 *   - the first call on a device looks up the array's device address (a
 *     set-up step, repeated for a context not seen before, e.g. after
 *     cudaDeviceReset); make that first call before any stream capture;
 *   - all calls share the array, so calls that overlap on the GPU (for
 *     example on two streams at once) race; each call writes every partial
 *     it reads, so nothing needs clearing between calls;
 *   - gvol is still accumulated into: the caller zeroes it.
 * No counterpart in the reference, whose adjoint allocates its partials with
 * the torch allocator on every call. */
NDRR_API int32_t ndrr_raymarch_bwd_noalloc(const ndrr_raymarch_args* args, void* stream);

/* Empty-space sample windows ahead of the march. For the rays of `args`
 * (geometry, n_samples, optional t_window) and its skip_mode — OCCUPANCY:
 * the distance-field walk to the first and last occupied cell; PROPOSAL: the
 * learned network's interval, checked against the occupancy grid, with the
 * full box-culled window for rays that fail the check — writes each ray's
 * window [first sample, one past the last] to `windows` ([B, N, 2] int32,
 * device) and adds to args->skip_stats when set. A march given these windows
 * (args.sample_window, skip_mode 0) computes the same image and pose/camera
 * gradients as one that skips in-kernel; one call serves the forward and the
 * adjoint of a step. The network runs on the tensor cores (mma.sync, bf16
 * operands, fp32 accumulation) in a persistent kernel that stages its weights
 * in shared memory once per CTA. No counterpart in the reference. */
NDRR_API int32_t ndrr_skip_windows(const ndrr_raymarch_args* args, int32_t* windows, void* stream);

/* 3-D texture of a float32 volume [D, H, W] for the texture-filtered forward
 * variant: allocates a CUDA array (D x H x W floats), copies the volume on
 * `stream`, and creates a texture object with linear filtering and zero
 * border; *handle receives it. ndrr_texture_destroy frees both. */
NDRR_API int32_t ndrr_texture_create(const float* vol, int32_t D, int32_t H, int32_t W, uint64_t* handle,
                                     void* stream);
NDRR_API int32_t ndrr_texture_destroy(uint64_t handle);

/* ---- intrinsics resample ---------------------------------------------------- *
 * Replaces the reference's camera/homography.py:6-58 `resample`: each
 * destination pixel (x, y) of image b samples the source image at
 * hom_b (x, y, 1) (perspective divide), bilinearly with align_corners
 * semantics and zero padding. img/out: [B, C, H, W] float32, contiguous;
 * hom: [B, 3, 3] float32 = K_old K_new^-1 (the caller forms it from the two
 * inverse intrinsics). */
NDRR_API int32_t ndrr_homography_resample(const float* img, const float* hom, int32_t B, int32_t C, int32_t H,
                                          int32_t W, float* out, void* stream);

/* Scratch bytes of ndrr_homography_resample_bwd (per-CTA partials of the
 * homography gradient). */
NDRR_API int32_t ndrr_homography_resample_bwd_workspace_bytes(int32_t B, int32_t H, int32_t W, uint64_t* bytes);

/* Adjoint of ndrr_homography_resample for the upstream gradient go: gimg
 * ([B, C, H, W], ACCUMULATED into with atomics, zero it first; or NULL) and
 * ghom ([B, 3, 3], written, deterministic fixed-order reduction; or NULL). */
NDRR_API int32_t ndrr_homography_resample_bwd(const float* go, const float* img, const float* hom, int32_t B,
                                              int32_t C, int32_t H, int32_t W, float* gimg, float* ghom,
                                              void* workspace, uint64_t workspace_bytes, void* stream);

/* ---- normalised cross-correlation ------------------------------------------ *
 * Replaces the reference's metrics/ncc.py:8-37 NormalizedCrossCorrelation2d
 * (the image-similarity loss of a registration step). x1, x2: [B, P, N]
 * float32, contiguous: B batch elements of P planes of N pixels (P = C image
 * channels, or C x patches when the caller unfolds local windows into
 * planes). Each plane of each image is centred and divided by
 * sqrt(population variance + eps); score[b] = sum over its planes and pixels
 * of the products / (P N). stats: [B, P, NDRR_NCC_STATS] float32, written
 * by the forward and read by the adjoint; workspace: the forward's per-chunk
 * moments (ndrr_ncc_workspace_bytes). */
#define NDRR_NCC_STATS 8
NDRR_API int32_t ndrr_ncc_workspace_bytes(int32_t B, int32_t P, int32_t N, uint64_t* bytes);
NDRR_API int32_t ndrr_ncc_fwd(const float* x1, const float* x2, int32_t B, int32_t P, int32_t N, float eps,
                              float* score, float* stats, void* workspace, uint64_t workspace_bytes,
                              void* stream);

/* Adjoint for the upstream gradient go [B]: g1 = d/dx1, g2 = d/dx2 ([B, P, N],
 * written; either may be NULL). */
NDRR_API int32_t ndrr_ncc_bwd(const float* go, const float* x1, const float* x2, const float* stats, int32_t B,
                              int32_t P, int32_t N, float* g1, float* g2, void* stream);

/* ---- registration pose ------------------------------------------------------ *
 * Replaces the reference's Registration.pose (registration/registration.py:
 * 64-68 with geometry/se3.py:179-221, "so3_log"): the pose of each batch
 * element is rt_inv @ pivot @ T @ pivot_inv with T = [[R, R xyz], [0, 1]] and
 * R = exp([rot]x) (Rodrigues). rot, xyz: [B or 1, 3] float32 (rows of a
 * single-row parameter are broadcast: pass param_rows 1); rt_inv, pivot,
 * pivot_inv, pose: [B, 4, 4] float32, contiguous. Evaluated in float64, one
 * thread per pose. */
NDRR_API int32_t ndrr_pose_so3_fwd(const float* rot, const float* xyz, int32_t param_rows, const float* rt_inv,
                                   const float* pivot, const float* pivot_inv, int32_t B, float* pose,
                                   void* stream);

/* Adjoint for gpose [B, 4, 4]: g_rot, g_xyz [B, 3] per pose (written; the
 * caller sums the rows for a broadcast parameter). */
NDRR_API int32_t ndrr_pose_so3_bwd(const float* gpose, const float* rot, const float* xyz, int32_t param_rows,
                                   const float* rt_inv, const float* pivot, const float* pivot_inv, int32_t B,
                                   float* g_rot, float* g_xyz, void* stream);

/* ---- persistent batched launch -------------------------------------------- *
 * Many render requests — different volumes (same dtype), detector sizes and
 * sample counts — marched by ONE persistent kernel: CTAs take (request, tile)
 * work items from an atomic counter until all are done, so small requests do
 * not leave the GPU idle and a whole batch is one launch (capturable in a CUDA
 * graph: the descriptors and their device buffers stay fixed while the poses
 * they point to change). Forward and pose/camera adjoint (no volume gradient).
 * No counterpart in the reference, which renders one volume and one detector
 * size per call. */
typedef struct ndrr_request {
    const void* vol;            /* [D, H, W] in the batch's vol_dtype          */
    const void* lab;            /* label map (batch lab_dtype) or NULL if C==1 */
    int32_t D, H, W;
    int32_t N;                  /* rays                                         */
    int32_t width;              /* detector width (rays form an image)          */
    int32_t n_samples;          /* >= 2                                         */
    int32_t src_per_ray;        /* 0: src [1, 3], 1: src [N, 3]                 */
    int32_t tile_w, tile_h, sample_split; /* tile_w * tile_h * sample_split == 256 */
    const float* M;             /* [3, 4] camera -> voxel                       */
    const float* src;
    const float* tgt;           /* [N, 3]                                       */
    const float* step;          /* [N]                                          */
    void* out;                  /* forward output [C, N] in vol_dtype           */
    const void* go;             /* adjoint input [C, N] in go_dtype             */
    float* gM;                  /* adjoint output [3, 4]                        */
    float* gsrc;                /* [1 | N, 3] when need_gcam                    */
    float* gtgt;                /* [N, 3] when need_gcam                        */
    float* gstep;               /* [N] when need_gcam                           */
    const void* vol_quad;       /* quad-layout copy of vol (ndrr_quad_build) or
                                   NULL: the request's samples read it instead
                                   of vol (same results)                        */
} ndrr_request;

typedef struct ndrr_batch_args {
    uint32_t struct_size;       /* sizeof(ndrr_batch_args)                      */
    uint32_t abi_version;
    const ndrr_request* requests;   /* DEVICE array [n_requests]               */
    const int32_t* tile_offsets;    /* DEVICE [n_requests + 1]: exclusive prefix
                                       sums of each request's tile count        */
    int32_t n_requests;
    int32_t total_tiles;
    int32_t vol_dtype, lab_dtype, go_dtype;
    int32_t n_classes;
    int32_t need_gcam;
    int32_t ctas;               /* persistent CTAs, 0 = library default        */
    void* workspace;            /* ndrr_batched_workspace_bytes                 */
    uint64_t workspace_bytes;
    int32_t reserved[4];
} ndrr_batch_args;

/* Host-side check of a request array before it is uploaded; also returns the
 * number of tiles of each request (tiles[n]) so the caller can build the
 * prefix sums. */
NDRR_API int32_t ndrr_batch_validate(const ndrr_request* host_requests, int32_t n_requests, int32_t n_classes,
                                     int32_t* tiles);
NDRR_API int32_t ndrr_batched_workspace_bytes(int32_t total_tiles, uint64_t* bytes);
NDRR_API int32_t ndrr_batched_fwd(const ndrr_batch_args* args, void* stream);
NDRR_API int32_t ndrr_batched_bwd(const ndrr_batch_args* args, void* stream);

/* ---- quad volume layout --------------------------------------------------- *
 * Element (qz, qy, qx) holds the corners (x0, y0), (x0+1, y0), (x0, y0+1),
 * (x0+1, y0+1) of plane z = qz - 2 with x0 = qx - 2, y0 = qy - 2, zeros
 * outside the volume; extent (D + 4) x (H + 3) x (W + 3); element size 16 B
 * for f32 volumes, 8 B for f16/bf16. No counterpart in the reference. */
NDRR_API int32_t ndrr_quad_dims(int32_t D, int32_t H, int32_t W, int32_t* qz, int32_t* qy, int32_t* qx);
NDRR_API int32_t ndrr_quad_build(const void* vol, int32_t vol_dtype, int32_t D, int32_t H, int32_t W, void* quad,
                                 void* stream);

/* Labelled quad layout of a 16-bit (f16 / bf16) volume and its label map
 * (any ndrr_dtype, truncated toward zero like a cast): the same extent, 16
 * bytes per element — the four corner values of ndrr_quad_build's 8-byte
 * element, then the four corners' classes as uint8 (a class in [0,
 * n_classes) as is, 255 for a label outside it, 0 for a corner outside the
 * volume), then 4 zero bytes. n_classes in 2..255. Use with quad_labels = 1.
 * No counterpart in the reference. */
NDRR_API int32_t ndrr_quad_build_labeled(const void* vol, int32_t vol_dtype, const void* lab, int32_t lab_dtype,
                                         int32_t n_classes, int32_t D, int32_t H, int32_t W, void* quad,
                                         void* stream);

/* HU -> linear attenuation (1/mm) of n elements, elementwise: replaces the
 * reference's hu_to_mu (src/nanodrr/data/preprocess.py:9-50), which Subject
 * .image applies (src/nanodrr/data/subject.py:98-107). hu and mu: n elements
 * of dtype (f32, f16 or bf16), device pointers; mu may alias hu. HU is
 * clamped at -1000; at or below 0 HU mu = (hu / 1000 + 1) * mu_water, above
 * it mu = mu_water + (hu / hu_bone) * (mu_bone - mu_water); mu is clamped at
 * 0. Computed in fp32. */
NDRR_API int32_t ndrr_hu_to_mu(const void* hu, int32_t dtype, int64_t n, float mu_water, float mu_bone,
                               float hu_bone, void* mu, void* stream);

/* Camera-space ray endpoints of a detector, one launch: replaces the
 * reference's _make_tgt / _make_src (src/nanodrr/drr/renderer.py:101-132).
 * k_inv: n_k (1 or batch) row-major 3x3 inverse intrinsics; sdd: n_s (1 or
 * batch) source-to-detector distances; all float32 device pointers.
 * tgt [batch, height*width, 3] = sdd * (K0 * (u + 0.5) + K1 * (v + 0.5) + K2)
 * for pixel n = v * width + u (Kc: column c of K^-1), each product and sum
 * rounded on its own, left to right, bitwise the reference's expression in
 * float32. src: [batch, 1, 3] zeros for a pinhole camera, or [batch,
 * height*width, 3] = tgt with z - sdd when orthographic != 0. batch must
 * equal max(n_k, n_s). No counterpart in the reference's C-level
 * interface. */
NDRR_API int32_t ndrr_camera_rays(const float* k_inv, int32_t n_k, const float* sdd, int32_t n_s, int32_t batch,
                                  int32_t height, int32_t width, int32_t orthographic, float* src, float* tgt,
                                  void* stream);

/* ---- measurement ------------------------------------------------------------ *
 * Kernel timing hook: while set, the calling thread's ray-march entry points
 * record `start` (a cudaEvent_t) on their stream just before each ray-march
 * kernel they launch and `stop` just after it, so cudaEventElapsedTime gives
 * the march kernel's own duration apart from the other launches of the same
 * call (gradient zeroing, slab planning, pose reduction, gradient fold).
 * ndrr_set_kernel_events(NULL, NULL) turns it off. With more than one march
 * kernel per call the events bracket the last one. */
NDRR_API int32_t ndrr_set_kernel_events(void* start, void* stop);

/* L2 read-bandwidth probe: streams `bytes` of `buf` (device, 16-byte
 * aligned, contents arbitrary) `passes` times with L2-only loads from 4 CTAs
 * of 512 threads per SM; time it with events around the call. A buffer well
 * below the L2 size is read from L2 after the first pass. `sink` (device, 4
 * bytes) is written only in a case real data does not reach. */
NDRR_API int32_t ndrr_l2_read_probe(const void* buf, uint64_t bytes, int32_t passes, uint32_t* sink, void* stream);

/* Reduction-throughput probe: the volume-gradient scatter's pattern alone.
 * `buf` (device, 16-byte aligned, >= 5 planes of 512 x 512 x 16 bytes, at
 * most 4096 planes) is read as quad-entry planes; every thread of 4 CTAs of
 * 512 per SM adds 1.0 to the four floats of two entries (planes z and z + 1
 * of its cell: two red.global.add.v4.f32) per iteration, `iters` times, each
 * warp an 8 x 4 patch of neighbouring cells. `launched_threads` receives the
 * thread count, so samples = threads x iters; time the call with events. A
 * buffer of a few tens of MiB stays in L2 and gives the ceiling the adjoint's
 * scatter is measured against. */
NDRR_API int32_t ndrr_reduce_probe(void* buf, uint64_t bytes, int32_t iters, int32_t* launched_threads, void* stream);

/* ---- empty-space structures ---------------------------------------------- */
typedef struct ndrr_occupancy_args {
    uint32_t struct_size;   /* sizeof(ndrr_occupancy_args) */
    uint32_t abi_version;
    const void* vol;        /* [D, H, W] f32 / f16 / bf16 */
    int32_t vol_dtype;
    int32_t D, H, W;
    int32_t cell;           /* cell edge in voxels, 2..64 */
    int32_t max_dist;       /* Chebyshev distance cap in cells, 1..255 */
    uint8_t* grid;          /* [gz, gy, gx] output (ndrr_occupancy_dims) */
    uint8_t* scratch;       /* [gz, gy, gx] scratch */
} ndrr_occupancy_args;

/* Grid extent for a volume: ceil(dim / cell) + 2 cells per axis (one border
 * cell on each side). */
NDRR_API int32_t ndrr_occupancy_dims(int32_t D, int32_t H, int32_t W, int32_t cell, int32_t* gz, int32_t* gy,
                                     int32_t* gx);

/* Build the occupancy / distance grid of a volume. Grid cell g spans voxels
 * [(g - 1) cell, g cell) per axis and is occupied when any voxel within two
 * voxels of it is non-zero; the grid stores the Chebyshev distance in cells
 * to the nearest occupied cell (0 = occupied, capped at max_dist). No
 * counterpart in the reference, which marches every box-culled sample. */
NDRR_API int32_t ndrr_occupancy_build(const ndrr_occupancy_args* args, void* stream);

/* ---- learned proposal network ---------------------------------------------
 * 3-layer MLP 64 -> 64 -> 64 -> 2 on Fourier-encoded ray entry/exit points,
 * predicting the fractions of the in-box segment where a ray's non-empty
 * interval starts and ends. fp32 master parameters (NDRR_PROPOSAL_PARAMS
 * floats: W1 [64][64], b1, W2 [64][64], b2, W3 [2][64], b3) are trained by the
 * kernels below and packed to bf16 (NDRR_PROPOSAL_PACKED_BYTES) for the
 * tensor-core inference in the window kernel (ndrr_skip_windows). No
 * counterpart in the reference. */
#define NDRR_PROPOSAL_PARAMS 8450
#define NDRR_PROPOSAL_PACKED_BYTES 17952
#define NDRR_PROPOSAL_FEATURES 64

NDRR_API const char* ndrr_proposal_last_error(void);

/* Features [B*N, 64] f32, targets [B*N, 2] f32 and valid [B*N] u8 for the rays
 * described by `rays` (M, src, tgt, volume dims), from the per-ray non-empty
 * interval `extent` [B, N, 2] that ndrr_raymarch_fwd writes to out_extent,
 * widened by `widen_voxels` of Chebyshev distance on each side (use the
 * occupancy cell size + 3 so that the check can confirm a correct proposal). */
NDRR_API int32_t ndrr_proposal_dataset(const ndrr_raymarch_args* rays, const float* extent, float widen_voxels,
                                       float* features, float* targets, uint8_t* valid, void* stream);

/* Forward, asymmetric loss (clipping the target interval costs `alpha` times
 * more than widening it; for an empty target, t0 > t1, only a proposed
 * non-empty window costs) and backward over n rays; ACCUMULATES the gradient
 * of inv_count * sum(loss) into grads [NDRR_PROPOSAL_PARAMS] and the loss
 * into *loss. */
NDRR_API int32_t ndrr_proposal_train_step(const float* params, const float* features, const float* targets,
                                          const uint8_t* valid, int64_t n, float alpha, float inv_count,
                                          float* grads, float* loss, void* stream);

/* fp32 network outputs [n, 2]. */
NDRR_API int32_t ndrr_proposal_forward(const float* params, const float* features, int64_t n, float* out,
                                       void* stream);

/* One Adam update of the master parameters (step >= 1 for bias correction). */
NDRR_API int32_t ndrr_proposal_adam(float* params, const float* grads, float* m1, float* m2, int32_t step, float lr,
                                    float beta1, float beta2, float eps, void* stream);

/* Pack the fp32 master parameters into the bf16 inference layout. */
NDRR_API int32_t ndrr_proposal_pack(const float* params, void* packed, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NANODRR_GB300_H */
