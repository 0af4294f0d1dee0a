// extern "C" entry points: argument validation, launch-shape selection and
// error reporting. Validation mirrors the reference's host-side checks
// (n_samples >= 2 at nanodrr src/nanodrr/drr/renderer.py:71-72, the int32
// indexing limits of fused_supported at src/nanodrr/drr/backends.py:66-69)
// and adds the pointer/dtype/shape checks a C caller needs. Nothing here
// allocates device memory or synchronises.
#include <cuda.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "ndrr_march.cuh"

namespace {

thread_local std::string g_last_error;

int32_t fail(int32_t code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int32_t ok() {
    g_last_error.clear();
    return NDRR_OK;
}

bool is_float_dtype(int32_t d) { return d == NDRR_F32 || d == NDRR_F16 || d == NDRR_BF16; }
bool is_any_dtype(int32_t d) { return d >= NDRR_F32 && d <= NDRR_I64; }

constexpr long long kInt32Max = 2147483647LL;
constexpr int kMaxBlock = 512;
constexpr size_t kMaxSmem = 227 * 1024;

int sm_count_current() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return 148;
    return sms;
}

size_t dtype_bytes(int32_t d) {
    switch (d) {
        case NDRR_F32: case NDRR_I32: return 4;
        case NDRR_F16: case NDRR_BF16: case NDRR_I16: return 2;
        case NDRR_I64: return 8;
        default: return 1;
    }
}

bool misaligned(const void* p, size_t align) { return (reinterpret_cast<uintptr_t>(p) % align) != 0; }

// Alignment of every pointer the kernels dereference: each element type's
// natural alignment, and 16 bytes for the arrays read or written with
// 16-byte vector instructions (the quad layout, its gradient scratch, and
// the volume gradient the quad fold writes four floats at a time). A
// misaligned vector access would end the CUDA context, so it is refused
// here, before any launch.
int32_t validate_alignment(const ndrr_raymarch_args* a) {
    struct Check {
        const void* p;
        size_t align;
        const char* name;
    };
    const size_t ve = dtype_bytes(a->vol_dtype);
    const Check checks[] = {
        {a->vol, ve, "vol"},
        {a->n_classes > 1 ? a->lab : nullptr, dtype_bytes(a->lab_dtype), "lab"},
        {a->M, 4, "M"},
        {a->M_lo, 4, "M_lo"},
        {a->src, 4, "src"},
        {a->tgt, 4, "tgt"},
        {a->step, 4, "step"},
        {a->t_window, 4, "t_window"},
        {a->out, dtype_bytes(a->out_dtype), "out"},
        {a->out_total, dtype_bytes(a->out_dtype), "out_total"},
        {a->go, dtype_bytes(a->go_dtype), "go"},
        {a->gvol, a->vol_quad != nullptr ? 16 : 4, "gvol (16 bytes with the quad layout)"},
        {a->gM, 4, "gM"},
        {a->gsrc, 4, "gsrc"},
        {a->gtgt, 4, "gtgt"},
        {a->gstep, 4, "gstep"},
        {a->workspace, 16, "workspace"},
        {a->skip_stats, 8, "skip_stats"},
        {a->out_extent, 8, "out_extent"},
        {a->vol_quad, 16, "vol_quad"},
        {a->gvol_quad, 16, "gvol_quad"},
        {a->sample_window, 8, "sample_window"},
    };
    for (const Check& c : checks)
        if (c.p != nullptr && misaligned(c.p, c.align))
            return fail(NDRR_ERR_INVALID_ARGUMENT, "%s must be %zu-byte aligned (got %p)", c.name, c.align, c.p);
    return NDRR_OK;
}

// Shape/pointer checks shared by the forward and the adjoint.
int32_t validate_common(const ndrr_raymarch_args* a) {
    if (a == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "args is NULL");
    if (a->struct_size != sizeof(ndrr_raymarch_args))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "struct_size %u does not match the library's %zu", a->struct_size,
                    sizeof(ndrr_raymarch_args));
    if (a->abi_version != NDRR_ABI_VERSION)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "abi_version %u, library is %d", a->abi_version, NDRR_ABI_VERSION);
    if (a->n_samples < 2) return fail(NDRR_ERR_INVALID_ARGUMENT, "n_samples must be at least 2 (got %d)", a->n_samples);
    if (a->B < 0 || a->N < 0) return fail(NDRR_ERR_INVALID_ARGUMENT, "negative batch (%d) or ray count (%d)", a->B, a->N);
    if (a->D < 1 || a->H < 1 || a->W < 1)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "volume dims must be positive (got %d x %d x %d)", a->D, a->H, a->W);
    if (!is_float_dtype(a->vol_dtype))
        return fail(NDRR_ERR_DTYPE, "volume dtype %d unsupported (f32, f16, bf16)", a->vol_dtype);
    if (a->vol == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "vol is NULL");
    const long long numel = (long long)a->D * a->H * a->W;
    if (numel >= kInt32Max)
        return fail(NDRR_ERR_LIMIT, "volume has %lld voxels; the kernels index with int32 (< 2^31)", numel);
    if (a->n_classes < 1) return fail(NDRR_ERR_INVALID_ARGUMENT, "n_classes must be >= 1 (got %d)", a->n_classes);
    if (a->n_classes > 1) {
        if (a->lab == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "n_classes > 1 needs a label map");
        if (!is_any_dtype(a->lab_dtype)) return fail(NDRR_ERR_DTYPE, "label dtype %d unsupported", a->lab_dtype);
    }
    if (a->B == 0 || a->N == 0) return NDRR_OK;
    if (a->M == nullptr || a->src == nullptr || a->tgt == nullptr || a->step == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "M, src, tgt and step must be non-NULL");
    const long long BN = (long long)a->B * a->N;
    if ((long long)a->n_classes * BN >= kInt32Max || 3 * BN >= kInt32Max)
        return fail(NDRR_ERR_LIMIT, "C*B*N = %lld and 3*B*N = %lld must stay below 2^31",
                    (long long)a->n_classes * BN, 3 * BN);
    if (a->tile_w != 0 && (a->tile_w % 8 != 0 || a->tile_w < 8 || a->tile_w > 64))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "tile_w must be a multiple of 8 in [8, 64] (got %d)", a->tile_w);
    if (a->tile_h != 0 && (a->tile_h % 4 != 0 || a->tile_h < 4 || a->tile_h > 64))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "tile_h must be a multiple of 4 in [4, 64] (got %d)", a->tile_h);
    if (a->sample_split != 0 && a->sample_split != 1 && a->sample_split != 2 && a->sample_split != 4 &&
        a->sample_split != 8 && a->sample_split != 16)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "sample_split must be 1, 2, 4, 8 or 16 (got %d)", a->sample_split);
    if (a->skip_mode < NDRR_SKIP_NONE || a->skip_mode > NDRR_SKIP_PROPOSAL)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "skip_mode must be 0, 1 or 2 (got %d)", a->skip_mode);
    if (a->skip_mode != NDRR_SKIP_NONE) {
        if (a->occ_grid == nullptr || a->occ_cell < 2 || a->occ_cell > 64)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "skipping needs an occupancy grid with a cell of 2..64 voxels");
        const int gx = (a->W + a->occ_cell - 1) / a->occ_cell + 2, gy = (a->H + a->occ_cell - 1) / a->occ_cell + 2,
                  gz = (a->D + a->occ_cell - 1) / a->occ_cell + 2;
        if (a->occ_gx != gx || a->occ_gy != gy || a->occ_gz != gz)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "occupancy grid %dx%dx%d does not match the volume (%dx%dx%d)",
                        a->occ_gz, a->occ_gy, a->occ_gx, gz, gy, gx);
        if (a->skip_mode == NDRR_SKIP_PROPOSAL && a->proposal_params == nullptr)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "proposal skipping needs packed proposal parameters");
        if (!(a->proposal_margin >= 0.f)) return fail(NDRR_ERR_INVALID_ARGUMENT, "proposal_margin must be >= 0");
    }
    if (validate_alignment(a) != NDRR_OK) return NDRR_ERR_INVALID_ARGUMENT;
    if (a->sample_window != nullptr && a->skip_mode != NDRR_SKIP_NONE)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "sample_window and skip_mode are exclusive (one skip at a time)");
    if (a->vol_quad != nullptr && (long long)(a->D + 4) * (a->H + 3) * (a->W + 3) >= kInt32Max)
        return fail(NDRR_ERR_LIMIT, "quad layout of a %dx%dx%d volume exceeds int32 indexing", a->D, a->H, a->W);
    if (a->gvol_overwrite != 0 && (a->gvol_overwrite != 1 || a->vol_quad == nullptr))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "gvol_overwrite is 0, or 1 with the quad layout");
    if (a->fwd_mode != NDRR_FWD_DEFAULT && a->fwd_mode != NDRR_FWD_TMA)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "fwd_mode must be 0 or 1 (got %d)", a->fwd_mode);
    if (a->gvol_mode < NDRR_GVOL_AUTO || a->gvol_mode > NDRR_GVOL_SPLIT)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "gvol_mode must be 0 .. 5 (got %d)", a->gvol_mode);
    if ((a->gvol_mode == NDRR_GVOL_SLAB || a->gvol_mode == NDRR_GVOL_SLAB_WARP || a->gvol_mode == NDRR_GVOL_SPLIT) &&
        a->vol_quad == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "gvol_mode 3 and 4 (slab-ordered) need the quad layout (vol_quad)");
    if (a->brick_cap < 0 || a->brick_cap > 56 * 1024)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "brick capacity %d out of range [0, 57344] voxels", a->brick_cap);
    if (a->slab_mib < 0 || a->slab_mib > 4096)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "slab size %d MiB out of range [0, 4096]", a->slab_mib);
    if (a->quad_labels != 0) {
        if (a->quad_labels != 1 || a->vol_quad == nullptr)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "quad_labels is 0, or 1 with a labelled quad in vol_quad");
        if (a->vol_dtype == NDRR_F32 || a->n_classes < 2 || a->n_classes > 255)
            return fail(NDRR_ERR_INVALID_ARGUMENT,
                        "the labelled quad layout is for f16/bf16 volumes with n_classes in 2..255");
    }
    return NDRR_OK;
}

int32_t validate_shape(const ndrr::LaunchShape& ls, size_t smem) {
    const int block = ls.tw * ls.th * ls.K;
    if (block > kMaxBlock || (block % 32) != 0)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "tile %dx%d with sample_split %d gives %d threads (max %d)", ls.tw,
                    ls.th, ls.K, block, kMaxBlock);
    if (smem > kMaxSmem)
        return fail(NDRR_ERR_LIMIT, "launch needs %zu bytes of shared memory (max %zu); reduce n_classes or the tile",
                    smem, kMaxSmem);
    return NDRR_OK;
}

// The learned proposal runs in the window kernel only (ndrr_skip_windows).
int32_t reject_proposal_march(const ndrr_raymarch_args* a) {
    if (a->skip_mode == NDRR_SKIP_PROPOSAL)
        return fail(NDRR_ERR_INVALID_ARGUMENT,
                    "skip_mode 2 (proposal) is computed by ndrr_skip_windows: pass its windows as sample_window");
    return NDRR_OK;
}

}  // namespace

extern "C" {

int32_t ndrr_abi_version(void) { return NDRR_ABI_VERSION; }

const char* ndrr_build_info(void) {
    return "nanodrr_gb300 abi " "3" " sm_103a nvcc " __DATE__;
}

const char* ndrr_last_error(void) { return g_last_error.c_str(); }

int32_t ndrr_device_flags(uint32_t* flags, int32_t clear) {
    if (flags == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "flags is NULL");
    unsigned v = 0;
    const cudaError_t e = ndrr::device_flags(&v, clear != 0);
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "reading the device flags failed: %s", cudaGetErrorString(e));
    *flags = v;
    return ok();
}

int32_t ndrr_raymarch_fwd(const ndrr_raymarch_args* a, void* stream) {
    int32_t rc = validate_common(a);
    if (rc == NDRR_OK) rc = reject_proposal_march(a);
    if (rc != NDRR_OK) return rc;
    if (a->B == 0 || a->N == 0) return ok();
    if (a->out == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "out is NULL");
    if (!is_float_dtype(a->out_dtype)) return fail(NDRR_ERR_DTYPE, "out dtype %d unsupported", a->out_dtype);
    if (a->skip_mode != NDRR_SKIP_NONE && a->out_dtype != a->vol_dtype)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "empty-space skipping writes the output in the volume's dtype");
    if (a->vol_quad != nullptr && a->out_dtype != a->vol_dtype)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "the quad layout writes the output in the volume's dtype");
    const ndrr::LaunchShape ls = ndrr::choose_shape(*a, sm_count_current());
    if (a->fwd_mode == NDRR_FWD_TMA) {
        if (a->vol_dtype != NDRR_F32 || a->out_dtype != NDRR_F32 || a->W % 4 != 0 || a->n_classes != 1 ||
            a->skip_mode != NDRR_SKIP_NONE || a->vol_quad != nullptr || a->sample_window != nullptr ||
            a->out_total != nullptr || a->out_extent != nullptr || a->vol_texture != 0)
            return fail(NDRR_ERR_INVALID_ARGUMENT,
                        "the TMA forward takes an f32 volume with W a multiple of 4, f32 output, one channel, "
                        "no skipping, windows, quad layout, texture, total or extent output");
        if (reinterpret_cast<uintptr_t>(a->vol) % 16 != 0)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "the TMA forward needs a 16-byte aligned volume");
        const cudaError_t e = ndrr::launch_fwd_tma(*a, ls, reinterpret_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "TMA forward launch failed: %s", cudaGetErrorString(e));
        return ok();
    }
    if (a->vol_texture != 0) {
        if (a->n_classes != 1 || a->skip_mode != NDRR_SKIP_NONE || a->vol_quad != nullptr ||
            a->sample_window != nullptr || a->out_total != nullptr || a->out_extent != nullptr)
            return fail(NDRR_ERR_INVALID_ARGUMENT,
                        "the texture-filtered forward takes one channel, no skipping, windows, quad layout, total or "
                        "extent output");
        rc = validate_shape(ls, (size_t)ls.tw * ls.th * ls.K * sizeof(float));
        if (rc != NDRR_OK) return rc;
        const cudaError_t e = ndrr::launch_fwd_tex(*a, ls, reinterpret_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "texture forward launch failed: %s", cudaGetErrorString(e));
        return ok();
    }
    rc = validate_shape(ls, ndrr::fwd_smem_bytes(*a, ls));
    if (rc != NDRR_OK) return rc;
    const cudaError_t e = ndrr::launch_fwd(*a, ls, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "forward launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_raymarch_bwd_workspace_bytes(const ndrr_raymarch_args* a, uint64_t* bytes) {
    if (bytes == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "bytes is NULL");
    *bytes = 0;
    int32_t rc = validate_common(a);
    if (rc != NDRR_OK) return rc;
    if (a->B == 0 || a->N == 0) return ok();
    // The partial buffer depends on the tile shape only, not on the sample
    // split, so no device query is needed (this call never touches the GPU).
    const ndrr::LaunchShape ls = ndrr::choose_shape(*a, 0);
    *bytes = ndrr::bwd_workspace_bytes(*a, ls);
    return ok();
}

int32_t ndrr_raymarch_bwd(const ndrr_raymarch_args* a, void* stream) {
    int32_t rc = validate_common(a);
    if (rc != NDRR_OK) return rc;
    // the split adjoint's pose pass honours the skip like a pose-only adjoint;
    // the slab-ordered adjoint of one channel takes sample windows as gather
    // windows (outside them no corner is loaded; every sample is scattered)
    const ndrr::LaunchShape ls0 = ndrr::choose_shape(*a, 0);
    const bool split = a->need_gvol && ls0.split;
    const bool gated = a->need_gvol && ls0.slab && !ls0.split && a->n_classes == 1;
    if (!a->need_gvol || split) rc = reject_proposal_march(a);
    if (rc != NDRR_OK) return rc;
    if (a->B == 0 || a->N == 0) return ok();
    if (a->go == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "go is NULL");
    if (!is_float_dtype(a->go_dtype)) return fail(NDRR_ERR_DTYPE, "go dtype %d unsupported", a->go_dtype);
    if (a->gM == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "gM is NULL");
    if (a->need_gvol && a->gvol == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "need_gvol set but gvol is NULL");
    if (a->need_gvol && a->sample_window != nullptr && !split && !gated)
        return fail(NDRR_ERR_INVALID_ARGUMENT,
                    "sample_window with need_gvol needs the slab-ordered adjoint of one channel (gvol_mode 0, 3 or 4 "
                    "with the quad layout) or gvol_mode 5: the volume gradient needs every sample, and only those "
                    "use windows (to skip loads of zero corners)");
    if (a->need_gcam && (a->gsrc == nullptr || a->gtgt == nullptr || a->gstep == nullptr))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "need_gcam set but gsrc/gtgt/gstep is NULL");
    if (a->vol_quad != nullptr && a->need_gvol && a->gvol_quad == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "quad-layout adjoint with need_gvol needs gvol_quad scratch");
    // Workspace size depends on the tile shape only: check it before any
    // device query so a bad call fails without touching the GPU.
    const uint64_t need = ndrr::bwd_workspace_bytes(*a, ndrr::choose_shape(*a, 0));
    if (a->workspace == nullptr || a->workspace_bytes < need)
        return fail(NDRR_ERR_WORKSPACE, "adjoint needs %llu workspace bytes, got %llu", (unsigned long long)need,
                    (unsigned long long)(a->workspace ? a->workspace_bytes : 0));
    const ndrr::LaunchShape ls = ndrr::choose_shape(*a, sm_count_current());
    rc = validate_shape(ls, (a->need_gvol && ls.brick) ? ndrr::brick_smem_bytes(*a, ls) : ndrr::bwd_smem_bytes(*a, ls));
    if (rc != NDRR_OK) return rc;
    const cudaError_t e = ndrr::launch_bwd(*a, ls, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "adjoint launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_skip_windows(const ndrr_raymarch_args* a, int32_t* windows, void* stream) {
    int32_t rc = validate_common(a);
    if (rc != NDRR_OK) return rc;
    if (a->skip_mode != NDRR_SKIP_OCCUPANCY && a->skip_mode != NDRR_SKIP_PROPOSAL)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "skip windows need skip_mode 1 (occupancy) or 2 (proposal)");
    if (a->B == 0 || a->N == 0) return ok();
    if (windows == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "windows is NULL");
    if (reinterpret_cast<uintptr_t>(windows) % 8 != 0)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "windows must be 8-byte aligned");
    const cudaError_t e = ndrr::launch_skip_windows(*a, windows, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "skip-window launch failed: %s", cudaGetErrorString(e));
    return ok();
}

static int32_t homography_check(const float* img, const float* hom, int32_t B, int32_t C, int32_t H, int32_t W) {
    if (B < 0 || C < 1 || H < 2 || W < 2)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "resample needs B >= 0, C >= 1 and H, W >= 2 (got %d, %d, %d, %d)", B,
                    C, H, W);
    if ((long long)B * C * H * W >= kInt32Max * 4LL)
        return fail(NDRR_ERR_LIMIT, "resample of %d x %d x %d x %d pixels is too large", B, C, H, W);
    if (B > 65535) return fail(NDRR_ERR_LIMIT, "resample handles at most 65535 images per call (got %d)", B);
    if (B > 0 && (img == nullptr || hom == nullptr))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "img and hom must be non-NULL");
    return NDRR_OK;
}

int32_t ndrr_homography_resample(const float* img, const float* hom, int32_t B, int32_t C, int32_t H, int32_t W,
                                 float* out, void* stream) {
    int32_t rc = homography_check(img, hom, B, C, H, W);
    if (rc != NDRR_OK) return rc;
    if (B == 0) return ok();
    if (out == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "out is NULL");
    const cudaError_t e = ndrr::launch_homography_fwd(img, hom, B, C, H, W, out, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "resample launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_homography_resample_bwd_workspace_bytes(int32_t B, int32_t H, int32_t W, uint64_t* bytes) {
    if (bytes == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "bytes is NULL");
    if (B < 0 || H < 2 || W < 2) return fail(NDRR_ERR_INVALID_ARGUMENT, "bad resample shape");
    *bytes = (uint64_t)B * ndrr::homography_blocks(H, W) * 9 * sizeof(float);
    return ok();
}

int32_t ndrr_homography_resample_bwd(const float* go, const float* img, const float* hom, int32_t B, int32_t C,
                                     int32_t H, int32_t W, float* gimg, float* ghom, void* workspace,
                                     uint64_t workspace_bytes, void* stream) {
    int32_t rc = homography_check(img, hom, B, C, H, W);
    if (rc != NDRR_OK) return rc;
    if (B == 0) return ok();
    if (go == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "go is NULL");
    const uint64_t need = (uint64_t)B * ndrr::homography_blocks(H, W) * 9 * sizeof(float);
    if (ghom != nullptr && (workspace == nullptr || workspace_bytes < need))
        return fail(NDRR_ERR_WORKSPACE, "resample adjoint needs %llu workspace bytes, got %llu",
                    (unsigned long long)need, (unsigned long long)(workspace ? workspace_bytes : 0));
    const cudaError_t e = ndrr::launch_homography_bwd(go, img, hom, B, C, H, W, gimg, ghom,
                                                      reinterpret_cast<float*>(workspace),
                                                      reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "resample adjoint launch failed: %s", cudaGetErrorString(e));
    return ok();
}

static int32_t ncc_check(const float* x1, const float* x2, int32_t B, int32_t P, int32_t N, const float* stats) {
    if (B < 0 || P < 1 || N < 1)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "ncc needs B >= 0, P >= 1, N >= 1 (got %d, %d, %d)", B, P, N);
    if ((long long)B * P >= kInt32Max || (long long)B * P * N >= kInt32Max * 16LL)
        return fail(NDRR_ERR_LIMIT, "ncc of %d x %d planes of %d pixels is too large", B, P, N);
    if (B > 0 && (x1 == nullptr || x2 == nullptr || stats == nullptr))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "x1, x2 and stats must be non-NULL");
    return NDRR_OK;
}

int32_t ndrr_ncc_workspace_bytes(int32_t B, int32_t P, int32_t N, uint64_t* bytes) {
    if (bytes == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "bytes is NULL");
    if (B < 0 || P < 1 || N < 1) return fail(NDRR_ERR_INVALID_ARGUMENT, "bad ncc shape");
    *bytes = ndrr::ncc_workspace_bytes(B, P, N);
    return ok();
}

int32_t ndrr_ncc_fwd(const float* x1, const float* x2, int32_t B, int32_t P, int32_t N, float eps, float* score,
                     float* stats, void* workspace, uint64_t workspace_bytes, void* stream) {
    int32_t rc = ncc_check(x1, x2, B, P, N, stats);
    if (rc != NDRR_OK) return rc;
    if (!(eps >= 0.f)) return fail(NDRR_ERR_INVALID_ARGUMENT, "eps must be >= 0");
    if (B == 0) return ok();
    if (score == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "score is NULL");
    if ((long long)N > 65535LL * 4096) return fail(NDRR_ERR_LIMIT, "ncc planes hold at most 268 M pixels");
    const uint64_t need = ndrr::ncc_workspace_bytes(B, P, N);
    if (workspace == nullptr || workspace_bytes < need)
        return fail(NDRR_ERR_WORKSPACE, "ncc needs %llu workspace bytes, got %llu", (unsigned long long)need,
                    (unsigned long long)(workspace ? workspace_bytes : 0));
    const cudaError_t e = ndrr::launch_ncc_fwd(x1, x2, B, P, N, eps, score, stats, workspace,
                                               reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "ncc launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_ncc_bwd(const float* go, const float* x1, const float* x2, const float* stats, int32_t B, int32_t P,
                     int32_t N, float* g1, float* g2, void* stream) {
    int32_t rc = ncc_check(x1, x2, B, P, N, stats);
    if (rc != NDRR_OK) return rc;
    if (B == 0 || (g1 == nullptr && g2 == nullptr)) return ok();
    if (go == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "go is NULL");
    if ((long long)N > 65535LL * 4096) return fail(NDRR_ERR_LIMIT, "ncc planes hold at most 268 M pixels");
    const cudaError_t e =
        ndrr::launch_ncc_bwd(go, x1, x2, stats, B, P, N, g1, g2, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "ncc adjoint launch failed: %s", cudaGetErrorString(e));
    return ok();
}

static int32_t pose_check(const float* rot, const float* xyz, int32_t param_rows, const float* rt_inv,
                          const float* pivot, const float* pivot_inv, int32_t B) {
    if (B < 0) return fail(NDRR_ERR_INVALID_ARGUMENT, "B must be >= 0");
    if (B == 0) return NDRR_OK;
    if (!rot || !xyz || !rt_inv || !pivot || !pivot_inv)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "pose inputs must be non-NULL");
    if (param_rows != 1 && param_rows != B)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "param_rows must be 1 or B (%d), got %d", B, param_rows);
    return NDRR_OK;
}

int32_t ndrr_pose_so3_fwd(const float* rot, const float* xyz, int32_t param_rows, const float* rt_inv,
                          const float* pivot, const float* pivot_inv, int32_t B, float* pose, void* stream) {
    const int32_t rc = pose_check(rot, xyz, param_rows, rt_inv, pivot, pivot_inv, B);
    if (rc != NDRR_OK) return rc;
    if (B == 0) return ok();
    if (pose == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "pose is NULL");
    const cudaError_t e = ndrr::launch_pose_fwd(rot, xyz, param_rows, rt_inv, pivot, pivot_inv, B, pose,
                                                reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "pose launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_pose_so3_bwd(const float* gpose, const float* rot, const float* xyz, int32_t param_rows,
                          const float* rt_inv, const float* pivot, const float* pivot_inv, int32_t B, float* g_rot,
                          float* g_xyz, void* stream) {
    const int32_t rc = pose_check(rot, xyz, param_rows, rt_inv, pivot, pivot_inv, B);
    if (rc != NDRR_OK) return rc;
    if (B == 0) return ok();
    if (!gpose || !g_rot || !g_xyz) return fail(NDRR_ERR_INVALID_ARGUMENT, "gpose, g_rot and g_xyz must be non-NULL");
    const cudaError_t e = ndrr::launch_pose_bwd(gpose, rot, xyz, param_rows, rt_inv, pivot, pivot_inv, B, g_rot,
                                                g_xyz, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "pose adjoint launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_texture_create(const float* vol, int32_t D, int32_t H, int32_t W, uint64_t* handle, void* stream) {
    if (vol == nullptr || handle == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "vol and handle must be non-NULL");
    if (D < 1 || H < 1 || W < 1 || D > 16384 || H > 16384 || W > 16384)
        return fail(NDRR_ERR_LIMIT, "3-D texture extent %d x %d x %d outside [1, 16384]", D, H, W);
    unsigned long long h = 0;
    const cudaError_t e = ndrr::texture_create(vol, D, H, W, &h, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "texture creation failed: %s", cudaGetErrorString(e));
    *handle = h;
    return ok();
}

int32_t ndrr_texture_destroy(uint64_t handle) {
    bool known = false;
    const cudaError_t e = ndrr::texture_destroy(handle, &known);
    if (!known) return fail(NDRR_ERR_INVALID_ARGUMENT, "unknown texture handle");
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "texture destruction failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_quad_dims(int32_t D, int32_t H, int32_t W, int32_t* qz, int32_t* qy, int32_t* qx) {
    if (qz == nullptr || qy == nullptr || qx == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "NULL output");
    if (D < 1 || H < 1 || W < 1) return fail(NDRR_ERR_INVALID_ARGUMENT, "dims must be positive");
    if ((long long)(D + 4) * (H + 3) * (W + 3) >= kInt32Max)
        return fail(NDRR_ERR_LIMIT, "quad layout exceeds int32 indexing");
    *qz = D + 4;
    *qy = H + 3;
    *qx = W + 3;
    return ok();
}

int32_t ndrr_quad_build(const void* vol, int32_t dtype, int32_t D, int32_t H, int32_t W, void* quad, void* stream) {
    if (vol == nullptr || quad == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "vol and quad must be non-NULL");
    if (!is_float_dtype(dtype)) return fail(NDRR_ERR_DTYPE, "volume dtype %d unsupported", dtype);
    if (misaligned(quad, 16) || misaligned(vol, dtype_bytes(dtype)))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "quad must be 16-byte aligned and vol aligned to its element");
    int32_t qz, qy, qx;
    int32_t rc = ndrr_quad_dims(D, H, W, &qz, &qy, &qx);
    if (rc != NDRR_OK) return rc;
    const cudaError_t e = ndrr::launch_quad_build(vol, dtype, D, H, W, quad, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "quad build failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_quad_build_labeled(const void* vol, int32_t dtype, const void* lab, int32_t lab_dtype, int32_t n_classes,
                                int32_t D, int32_t H, int32_t W, void* quad, void* stream) {
    if (vol == nullptr || lab == nullptr || quad == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "vol, lab and quad must be non-NULL");
    if (dtype != NDRR_F16 && dtype != NDRR_BF16)
        return fail(NDRR_ERR_DTYPE, "the labelled quad layout takes f16 or bf16 volumes (got dtype %d)", dtype);
    if (!is_any_dtype(lab_dtype)) return fail(NDRR_ERR_DTYPE, "label dtype %d unsupported", lab_dtype);
    if (n_classes < 2 || n_classes > 255)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "n_classes must be 2..255 (got %d)", n_classes);
    if (misaligned(quad, 16) || misaligned(vol, 2) || misaligned(lab, dtype_bytes(lab_dtype)))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "quad must be 16-byte aligned, vol and lab aligned to their elements");
    int32_t qz, qy, qx;
    const int32_t rc = ndrr_quad_dims(D, H, W, &qz, &qy, &qx);
    if (rc != NDRR_OK) return rc;
    const cudaError_t e = ndrr::launch_quad_build_labeled(vol, dtype, lab, lab_dtype, n_classes, D, H, W, quad,
                                                          reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "labelled quad build failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_hu_to_mu(const void* hu, int32_t dtype, int64_t n, float mu_water, float mu_bone, float hu_bone,
                      void* mu, void* stream) {
    if (n < 0) return fail(NDRR_ERR_INVALID_ARGUMENT, "n must be >= 0 (got %lld)", (long long)n);
    if (!is_float_dtype(dtype)) return fail(NDRR_ERR_DTYPE, "HU dtype %d unsupported (f32, f16, bf16)", dtype);
    if (n == 0) return ok();
    if (hu == nullptr || mu == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "hu and mu must be non-NULL");
    if (!(hu_bone != 0.f)) return fail(NDRR_ERR_INVALID_ARGUMENT, "hu_bone must be non-zero");
    const float dmu = (float)((double)mu_bone - (double)mu_water);
    const cudaError_t e =
        ndrr::launch_hu_to_mu(hu, dtype, n, mu_water, dmu, hu_bone, mu, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "HU conversion launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_camera_rays(const float* k_inv, int32_t n_k, const float* sdd, int32_t n_s, int32_t batch,
                         int32_t height, int32_t width, int32_t orthographic, float* src, float* tgt, void* stream) {
    if (k_inv == nullptr || sdd == nullptr || src == nullptr || tgt == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "k_inv, sdd, src and tgt must be non-NULL");
    if (height < 1 || width < 1 || batch < 1)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "height, width and batch must be >= 1 (got %d, %d, %d)", height, width,
                    batch);
    if ((n_k != 1 && n_k != batch) || (n_s != 1 && n_s != batch) || batch != (n_k > n_s ? n_k : n_s))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "batch %d must be max(n_k, n_s) with each 1 or batch (n_k %d, n_s %d)", batch, n_k,
                    n_s);
    if ((long long)batch * height * width * 3 >= (1LL << 31))
        return fail(NDRR_ERR_LIMIT, "batch x pixels x 3 exceeds int32 indexing");
    if (misaligned(k_inv, 4) || misaligned(sdd, 4) || misaligned(src, 4) || misaligned(tgt, 4))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "k_inv, sdd, src and tgt must be 4-byte aligned");
    const cudaError_t e = ndrr::launch_camera_rays(k_inv, n_k, sdd, n_s, batch, height, width, orthographic != 0, src,
                                                   tgt, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "camera ray launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_set_kernel_events(void* start, void* stop) {
    if ((start == nullptr) != (stop == nullptr))
        return fail(NDRR_ERR_INVALID_ARGUMENT, "start and stop events are both set or both NULL");
    ndrr::KernelEvents& ev = ndrr::kernel_events();
    ev.start = reinterpret_cast<cudaEvent_t>(start);
    ev.stop = reinterpret_cast<cudaEvent_t>(stop);
    return ok();
}

int32_t ndrr_l2_read_probe(const void* buf, uint64_t bytes, int32_t passes, uint32_t* sink, void* stream) {
    if (buf == nullptr || sink == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "buf and sink must be non-NULL");
    if (misaligned(buf, 16) || bytes < 16 || passes < 1)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "the probe needs a 16-byte aligned buffer of >= 16 bytes, passes >= 1");
    const cudaError_t e = ndrr::launch_l2_probe(buf, bytes, passes, sink, sm_count_current(),
                                                reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "probe launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_reduce_probe(void* buf, uint64_t bytes, int32_t iters, int32_t* launched_threads, void* stream) {
    constexpr uint64_t kPlaneBytes = 512ull * 512ull * 16ull;
    if (buf == nullptr || launched_threads == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "buf and launched_threads must be non-NULL");
    if (misaligned(buf, 16) || bytes < 5 * kPlaneBytes || iters < 1)
        return fail(NDRR_ERR_INVALID_ARGUMENT,
                    "the reduction probe needs a 16-byte aligned buffer of at least 5 planes of 4 MiB, iters >= 1");
    const uint64_t planes = bytes / kPlaneBytes;
    if (planes > 4096) return fail(NDRR_ERR_INVALID_ARGUMENT, "the reduction probe takes at most 4096 planes");
    const int sms = sm_count_current();
    *launched_threads = (sms > 0 ? sms : 148) * 4 * 512;
    const cudaError_t e =
        ndrr::launch_reduce_probe(buf, (int)planes, iters, sms, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "reduction probe launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_batch_validate(const ndrr_request* q, int32_t n, int32_t n_classes, int32_t* tiles) {
    if (q == nullptr || tiles == nullptr || n < 0) return fail(NDRR_ERR_INVALID_ARGUMENT, "bad request array");
    if (n_classes < 1 || n_classes > 64) return fail(NDRR_ERR_INVALID_ARGUMENT, "batched n_classes must be 1..64");
    for (int32_t i = 0; i < n; ++i) {
        const ndrr_request& r = q[i];
        if (r.vol == nullptr || r.M == nullptr || r.src == nullptr || r.tgt == nullptr || r.step == nullptr)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "request %d: NULL geometry pointer", i);
        if (n_classes > 1 && r.lab == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "request %d: no label map", i);
        if (r.D < 1 || r.H < 1 || r.W < 1 || (long long)r.D * r.H * r.W >= kInt32Max)
            return fail(NDRR_ERR_INVALID_ARGUMENT, "request %d: bad volume dims", i);
        if (r.N < 1 || r.n_samples < 2) return fail(NDRR_ERR_INVALID_ARGUMENT, "request %d: N >= 1, n_samples >= 2", i);
        if ((long long)n_classes * r.N >= kInt32Max) return fail(NDRR_ERR_LIMIT, "request %d: C*N too large", i);
        if (r.tile_w % 8 || r.tile_h % 4 || r.tile_w < 8 || r.tile_h < 4 ||
            r.tile_w * r.tile_h * r.sample_split != 256 ||
            (r.sample_split != 1 && r.sample_split != 2 && r.sample_split != 4))
            return fail(NDRR_ERR_INVALID_ARGUMENT,
                        "request %d: tile_w (mult. of 8) * tile_h (mult. of 4) * sample_split (1/2/4) must be 256", i);
        if (misaligned(r.vol_quad, 16))
            return fail(NDRR_ERR_INVALID_ARGUMENT, "request %d: vol_quad must be 16-byte aligned", i);
        const ndrr::TileMap tm = ndrr::make_tilemap(r.N, r.width, r.tile_w, r.tile_h);
        tiles[i] = tm.tiles;
    }
    return ok();
}

int32_t ndrr_batched_workspace_bytes(int32_t total_tiles, uint64_t* bytes) {
    if (bytes == nullptr || total_tiles < 0) return fail(NDRR_ERR_INVALID_ARGUMENT, "bad argument");
    *bytes = 256 + (uint64_t)total_tiles * 16 * sizeof(float);
    return ok();
}

static int32_t batched_common(const ndrr_batch_args* a, bool backward, void* stream) {
    if (a == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "args is NULL");
    if (a->struct_size != sizeof(ndrr_batch_args) || a->abi_version != NDRR_ABI_VERSION)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "ndrr_batch_args size/version mismatch");
    if (a->n_requests == 0 || a->total_tiles == 0) return ok();
    if (a->n_requests < 0 || a->total_tiles < 0 || a->requests == nullptr || a->tile_offsets == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "requests / tile_offsets missing");
    if (!is_float_dtype(a->vol_dtype)) return fail(NDRR_ERR_DTYPE, "volume dtype %d unsupported", a->vol_dtype);
    if (a->n_classes < 1 || a->n_classes > 64) return fail(NDRR_ERR_INVALID_ARGUMENT, "n_classes must be 1..64");
    if (a->n_classes > 1 && !is_any_dtype(a->lab_dtype)) return fail(NDRR_ERR_DTYPE, "label dtype unsupported");
    if (backward && !is_float_dtype(a->go_dtype)) return fail(NDRR_ERR_DTYPE, "go dtype unsupported");
    uint64_t need = 0;
    ndrr_batched_workspace_bytes(a->total_tiles, &need);
    if (a->workspace == nullptr || a->workspace_bytes < need)
        return fail(NDRR_ERR_WORKSPACE, "batched launch needs %llu workspace bytes", (unsigned long long)need);
    const cudaError_t e = ndrr::launch_batched(*a, backward, sm_count_current(), reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "batched launch failed: %s", cudaGetErrorString(e));
    return ok();
}

int32_t ndrr_batched_fwd(const ndrr_batch_args* a, void* stream) { return batched_common(a, false, stream); }

int32_t ndrr_batched_bwd(const ndrr_batch_args* a, void* stream) { return batched_common(a, true, stream); }

int32_t ndrr_occupancy_dims(int32_t D, int32_t H, int32_t W, int32_t cell, int32_t* gz, int32_t* gy, int32_t* gx) {
    if (gz == nullptr || gy == nullptr || gx == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "NULL output");
    if (D < 1 || H < 1 || W < 1 || cell < 2 || cell > 64)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "dims must be positive and cell in 2..64");
    *gz = (D + cell - 1) / cell + 2;
    *gy = (H + cell - 1) / cell + 2;
    *gx = (W + cell - 1) / cell + 2;
    return ok();
}

int32_t ndrr_occupancy_build(const ndrr_occupancy_args* a, void* stream) {
    if (a == nullptr) return fail(NDRR_ERR_INVALID_ARGUMENT, "args is NULL");
    if (a->struct_size != sizeof(ndrr_occupancy_args) || a->abi_version != NDRR_ABI_VERSION)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "ndrr_occupancy_args size/version mismatch");
    if (a->vol == nullptr || a->grid == nullptr || a->scratch == nullptr)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "vol, grid and scratch must be non-NULL");
    if (!is_float_dtype(a->vol_dtype)) return fail(NDRR_ERR_DTYPE, "volume dtype %d unsupported", a->vol_dtype);
    if (a->D < 1 || a->H < 1 || a->W < 1 || (long long)a->D * a->H * a->W >= kInt32Max)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "bad volume dims");
    if (a->cell < 2 || a->cell > 64) return fail(NDRR_ERR_INVALID_ARGUMENT, "cell must be 2..64 (got %d)", a->cell);
    if (a->max_dist < 1 || a->max_dist > 255)
        return fail(NDRR_ERR_INVALID_ARGUMENT, "max_dist must be 1..255 (got %d)", a->max_dist);
    const cudaError_t e = ndrr::launch_occupancy(a->vol, a->vol_dtype, a->D, a->H, a->W, a->cell, a->max_dist,
                                                 a->grid, a->scratch, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "occupancy build failed: %s", cudaGetErrorString(e));
    return ok();
}

}  // extern "C"

// ===================================================== allocation-free adjoint
// Some callers cannot allocate device memory where they run the adjoint:
// hosts that own all device memory through their own pool and give plugins
// no allocator (inference servers, engines with a fixed device budget), and
// real-time loops where a cudaMalloc, with its implicit synchronisation and
// unbounded latency, is not allowed. They still pass inputs and outputs; the
// one scratch buffer the adjoint needs (the per-tile pose partials) lives in
// the file-scope device array below, which every GPU that loads this library
// holds until the process exits.
namespace {

// 4 MiB: 16 floats per (pose, detector tile); with the default 16 x 8 ray
// tile that is room for 65536 (pose, tile) pairs, e.g. 128 poses of 256 x 256.
constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The runtime can tear a device's context down and build a new one
// (cudaDeviceReset), which loads this module again, possibly at another
// address; a user can also make a context of their own current. So the
// looked-up address is kept per (device, context id) — context ids are never
// reused within a process — and looked up again for a context not seen
// before. The context id comes from the driver entry points cuCtxGetCurrent
// and cuCtxGetId, fetched through the runtime (no link to the driver
// library); without them every call looks the address up.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct CtxEntryPoints {
    CtxGetCurrentFn get_current = nullptr;
    CtxGetIdFn get_id = nullptr;
};

const CtxEntryPoints& ctx_entry_points() {
    static const CtxEntryPoints fns = []() {
        CtxEntryPoints f;
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qb == cudaDriverEntryPointSuccess) {
            f.get_current = reinterpret_cast<CtxGetCurrentFn>(a);
            f.get_id = reinterpret_cast<CtxGetIdFn>(b);
        }
        return f;
    }();
    return fns;
}

// Id of the calling thread's current context; false when none is current
// yet or the entry points are unavailable.
bool current_context_id(unsigned long long* id) {
    const CtxEntryPoints& f = ctx_entry_points();
    if (f.get_current == nullptr || f.get_id == nullptr) return false;
    CUcontext ctx = nullptr;
    if (f.get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return f.get_id(ctx, id) == CUDA_SUCCESS;
}

struct ScratchAddress {
    int device;
    unsigned long long context;
    void* ptr;
};

constexpr int kNoAllocMaxEntries = 64;
std::mutex g_noalloc_mu;
ScratchAddress g_noalloc_seen[kNoAllocMaxEntries];
int g_noalloc_count = 0;

// Device address of the scratch array in the current context. The host-side
// name of a __device__ array is only a stand-in, so the address is looked up
// with cudaGetSymbolAddress once per device and context, with that device
// current (the lookup also makes the device's primary context current when
// the thread has none yet).
cudaError_t noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    unsigned long long ctx = 0;
    bool known = current_context_id(&ctx);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (known) {
        for (int i = 0; i < g_noalloc_count; ++i) {
            if (g_noalloc_seen[i].device == dev && g_noalloc_seen[i].context == ctx) {
                *out = g_noalloc_seen[i].ptr;
                return cudaSuccess;
            }
        }
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (!known) known = current_context_id(&ctx);
    if (known) {
        // A full table overwrites a slot chosen by the context id (a lookup is cheap).
        const int slot = g_noalloc_count < kNoAllocMaxEntries ? g_noalloc_count++ : (int)(ctx % kNoAllocMaxEntries);
        g_noalloc_seen[slot] = ScratchAddress{dev, ctx, p};
    }
    *out = p;
    return cudaSuccess;
}

}  // namespace

extern "C" int32_t ndrr_raymarch_bwd_noalloc(const ndrr_raymarch_args* a, void* stream) {
    int32_t rc = validate_common(a);
    if (rc != NDRR_OK) return rc;
    if (a->B == 0 || a->N == 0) return ok();
    // The automatic volume-gradient mode would pick the slab-ordered adjoint,
    // whose work list does not fit the fixed scratch: use direct scatter.
    ndrr_raymarch_args local = *a;
    if (local.gvol_mode == NDRR_GVOL_AUTO) local.gvol_mode = NDRR_GVOL_DIRECT;
    const uint64_t need = ndrr::bwd_workspace_bytes(local, ndrr::choose_shape(local, 0));
    if (need > kNoAllocScratchBytes)
        return fail(NDRR_ERR_LIMIT,
                    "the allocation-free adjoint holds %llu bytes of scratch but this call needs %llu "
                    "(16 floats per pose and detector tile, more with gvol_mode 3); use fewer poses per call, "
                    "a larger tile, or ndrr_raymarch_bwd with a caller-provided workspace",
                    (unsigned long long)kNoAllocScratchBytes, (unsigned long long)need);
    void* scratch = nullptr;
    const cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) return fail(NDRR_ERR_CUDA, "scratch address lookup failed: %s", cudaGetErrorString(e));
    local.workspace = scratch;
    local.workspace_bytes = kNoAllocScratchBytes;
    return ndrr_raymarch_bwd(&local, stream);
}
