// Host-side launch planning shared by the ray-march launchers: kernel
// parameters, launch shape (tile, sample split, brick), shared-memory and
// workspace sizes.
#include "ndrr_march.cuh"

namespace ndrr {

MarchParams make_params(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    MarchParams p{};
    p.vol = a.vol;
    p.D = a.D;
    p.H = a.H;
    p.W = a.W;
    p.lab = a.lab;
    p.lab_dtype = a.lab_dtype;
    p.C = a.n_classes;
    p.M = a.M;
    p.M_lo = a.M_lo;
    p.src = a.src;
    p.tgt = a.tgt;
    p.step = a.step;
    p.src_per_ray = a.src_per_ray;
    p.B = a.B;
    p.N = a.N;
    p.S = a.n_samples;
    p.inv_s = 1.0f / (float)(a.n_samples - 1);
    p.t_window = a.t_window;
    p.win = a.sample_window;
    p.gwin = nullptr;
    p.out = a.out;
    p.out_total = a.out_total;
    p.go = a.go;
    p.go_dtype = a.go_dtype;
    p.gvol = a.gvol;
    p.gsrc = a.gsrc;
    p.gtgt = a.gtgt;
    p.gstep = a.gstep;
    p.partials = reinterpret_cast<float*>(a.workspace);
    p.skip_mode = a.skip_mode;
    p.occ.dist = a.occ_grid;
    p.occ.gx = a.occ_gx;
    p.occ.gy = a.occ_gy;
    p.occ.gz = a.occ_gz;
    p.occ.cell = a.occ_cell > 0 ? a.occ_cell : 1;
    p.proposal = reinterpret_cast<const unsigned char*>(a.proposal_params);
    p.margin = a.proposal_margin;
    p.stats = a.skip_stats;
    p.out_extent = a.out_extent;
    p.quad = a.vol_quad;
    p.gquad = a.gvol_quad;
    p.qg = make_quadgeom(a.D, a.H, a.W);
    p.tw = ls.tw;
    p.th = ls.th;
    p.K = ls.K;
    p.tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
    return p;
}

LaunchShape choose_shape(const ndrr_raymarch_args& a, int sm_count) {
    LaunchShape ls;
    ls.sm = sm_count;
    // A small launch (fewer than kSmallLaunchRays rays, e.g. one frame of a
    // 200^2 detector = 40 000 rays) takes narrow 8 x 4-ray tiles unless the
    // caller chose a tile: with 16 x 8 tiles split 4 ways one such frame was
    // 325 CTAs of 512 threads, at most two resident per SM, so 21 CTAs ran as
    // a second wave as long as the first; 8 x 4 tiles give 1250 CTAs of 128
    // threads, all resident at once. The rule depends on the ray count only,
    // never on the device, because the adjoint's workspace size (partials per
    // tile) is computed without a device query and must match the launch.
    constexpr double kSmallLaunchRays = 65536.0;
    const bool small = (double)a.B * a.N < kSmallLaunchRays && a.tile_w == 0 && a.tile_h == 0;
    ls.tw = a.tile_w > 0 ? a.tile_w : (small ? 8 : 16);
    ls.th = a.tile_h > 0 ? a.tile_h : (small ? 4 : 8);
    const TileMap tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
    const double threads = (double)a.B * tm.tiles * ls.tw * ls.th;
    const double want = (double)sm_count * 1024.0;
    if (a.sample_split > 0) {
        ls.K = a.sample_split;
    } else {
        // Split each ray's samples across threads only when the rays alone
        // leave the GPU under-filled (about 1024 resident threads per SM):
        // the smallest power of two up to 16 that reaches it.
        ls.K = 1;
        while (ls.K < 16 && threads * ls.K < want) ls.K *= 2;
        if (ls.tw * ls.th * ls.K > 512) ls.K = std::max(1, 512 / (ls.tw * ls.th));
    }
    // Volume-gradient scatter: direct global atomics by default; they
    // measured faster on GB300 than the per-slab shared-memory brick (whose
    // zero/flush passes and shared-memory atomics cost more than they save),
    // which stays available on request.
    ls.brick = a.gvol_mode == NDRR_GVOL_BRICK;
    if (ls.tw * ls.th > 256) ls.brick = false;  // brick kernel is built for <= 256 threads
    if (a.vol_quad != nullptr) ls.brick = false;  // the quad layout has its own scatter
    // Slab-ordered volume-gradient adjoint (the default for the quad layout
    // without camera gradients; measured 11 % faster than direct scatter at
    // 512^3 x 32 poses).
    ls.slab = (a.gvol_mode == NDRR_GVOL_SLAB || a.gvol_mode == NDRR_GVOL_SLAB_WARP ||
               a.gvol_mode == NDRR_GVOL_SPLIT || a.gvol_mode == NDRR_GVOL_AUTO) &&
              a.vol_quad != nullptr && a.need_gvol && !a.need_gcam;
    ls.split = ls.slab && a.gvol_mode == NDRR_GVOL_SPLIT && a.n_classes == 1;
    if (ls.brick) {
        ls.K = 1;
        const int nt = ls.tw * ls.th;
        ls.cap = a.brick_cap > 0 ? a.brick_cap : (nt <= 128 ? 12288 : 24576);
        ls.L0 = 16;
    }
    return ls;
}

size_t brick_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    const size_t NT = (size_t)ls.tw * ls.th;
    const size_t epi = std::max((NT / 32) * kPartialStride, a.need_gcam ? 7 * NT : (size_t)0);
    const size_t cap = std::max((size_t)ls.cap, epi);
    return cap * sizeof(float) + ((NT / 32) * 6 + 8) * sizeof(int);
}

uint64_t bwd_workspace_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    if (ls.slab) return slab_workspace_bytes(a, ls);
    const TileMap tm = make_tilemap(a.N, a.width, ls.tw, ls.th);
    return (uint64_t)a.B * tm.tiles * kPartialStride * sizeof(float);
}

// Forward: class accumulators and chunk partials, then the extent scratch.
size_t fwd_base_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    const size_t NT = (size_t)ls.tw * ls.th * ls.K;
    const size_t ext = a.out_extent ? 2 * NT : 0;
    return ((a.n_classes > 1 ? (size_t)a.n_classes + 1 : 1) * NT + ext) * sizeof(float);
}

size_t fwd_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) { return fwd_base_bytes(a, ls); }

// Adjoint: the epilogue scratch, then (proposal mode, persistent CTAs that
// keep the staged network across tiles) the network's region.
size_t bwd_epilogue_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) {
    const size_t NT = (size_t)ls.tw * ls.th * ls.K;
    const size_t wred = (NT / 32) * kPartialStride;
    const size_t cam = a.need_gcam ? 7 * NT : 0;
    return (std::max(wred, cam) * sizeof(float) + 15) & ~(size_t)15;
}

size_t bwd_smem_bytes(const ndrr_raymarch_args& a, const LaunchShape& ls) { return bwd_epilogue_bytes(a, ls); }

}  // namespace ndrr
