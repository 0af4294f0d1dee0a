"""Torch custom ops over the C ABI: `nanodrr_gb300::fused_raymarch` and
`nanodrr_gb300::fused_raymarch_bwd`.

Same schemas and argument meaning as the reference's ops
`nanodrr::fused_raymarch` (nanodrr src/nanodrr/drr/_fused.py:415-426) and
`nanodrr::fused_raymarch_bwd` (_fused.py:477-491), registered with fake
(meta) kernels for `torch.compile` (_fused.py:463, 534) and an autograd
formula (_fused.py:545-567). The work happens in `libnanodrr_gb300.so`; this
module only allocates outputs with the torch caching allocator, passes raw
pointers and the current stream, and maps C-ABI status codes to exceptions.

Differences from the reference, by design:
  - the forward writes its output in `vol.dtype` directly (no split-partials
    buffer and no separate sum/cast pass);
  - the backward returns `gsrc` already shaped like `src` (the reference's op
    returns per-ray `[B, N, 3]` and its autograd glue sums over rays when the
    source is shared, _fused.py:552-553; here that sum happens in-kernel).
"""

from __future__ import annotations

import ctypes

import torch

from . import _ffi

_TORCH_TO_NDRR = {
    torch.float32: _ffi.NDRR_F32,
    torch.float16: _ffi.NDRR_F16,
    torch.bfloat16: _ffi.NDRR_BF16,
    torch.uint8: _ffi.NDRR_U8,
    torch.bool: _ffi.NDRR_U8,
    torch.int8: _ffi.NDRR_I8,
    torch.int16: _ffi.NDRR_I16,
    torch.int32: _ffi.NDRR_I32,
    torch.int64: _ffi.NDRR_I64,
}
_FLOAT_DTYPES = (torch.float32, torch.float16, torch.bfloat16)


def ndrr_dtype(t: torch.Tensor) -> int:
    try:
        return _TORCH_TO_NDRR[t.dtype]
    except KeyError:
        raise ValueError(f"unsupported dtype {t.dtype}") from None


def _stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _ptr(t: torch.Tensor | None) -> int | None:
    if t is None or t.numel() == 0:
        return None
    return t.data_ptr()


def device_flags(clear: bool = False) -> int:
    """The library's device-side error flags on the current device
    (`_ffi.NDRR_FLAG_*`; e.g. a TMA-staged forward whose stage wait gave
    up). Synchronises the device."""
    lib = _ffi.load()
    v = ctypes.c_uint32(0)
    _ffi.check(lib.ndrr_device_flags(ctypes.byref(v), int(clear)), "ndrr_device_flags")
    return int(v.value)


def _check_inputs(vol, lab, M, src, tgt, step, n_samples, n_classes):
    if not vol.is_cuda:
        raise RuntimeError("nanodrr_gb300 renders on CUDA devices only (got a volume on %s)" % vol.device)
    if vol.dim() != 3:
        raise ValueError(f"vol must be [D, H, W], got shape {tuple(vol.shape)}")
    if vol.dtype not in _FLOAT_DTYPES:
        raise ValueError(f"vol dtype {vol.dtype} unsupported; use float32, float16 or bfloat16")
    if n_samples < 2:
        raise ValueError("n_samples must be at least 2")
    if tgt.dim() != 3 or tgt.shape[-1] != 3:
        raise ValueError(f"tgt must be [B, N, 3], got {tuple(tgt.shape)}")
    B, N, _ = tgt.shape
    if M.shape != (B, 3, 4):
        raise ValueError(f"M must be [B, 3, 4] = [{B}, 3, 4], got {tuple(M.shape)}")
    if src.dim() != 3 or src.shape[0] != B or src.shape[1] not in (1, N) or src.shape[2] != 3:
        raise ValueError(f"src must be [B, 1, 3] or [B, N, 3], got {tuple(src.shape)}")
    if step.shape != (B, N):
        raise ValueError(f"step must be [B, N] = [{B}, {N}], got {tuple(step.shape)}")
    if n_classes > 1 and lab.shape != vol.shape:
        raise ValueError(f"label map shape {tuple(lab.shape)} does not match the volume {tuple(vol.shape)}")
    for name, t in (("lab", lab), ("M", M), ("src", src), ("tgt", tgt), ("step", step)):
        if t.device != vol.device:
            raise ValueError(f"{name} is on {t.device}, the volume on {vol.device}")


def _base_args(vol, lab, M, src, tgt, step, n_samples, n_classes, width) -> _ffi.RaymarchArgs:
    B, N, _ = tgt.shape
    D, H, W = vol.shape
    a = _ffi.RaymarchArgs()
    a.vol = vol.data_ptr()
    a.vol_dtype = ndrr_dtype(vol)
    a.D, a.H, a.W = D, H, W
    a.n_classes = n_classes
    if n_classes > 1:
        a.lab = lab.data_ptr()
        a.lab_dtype = ndrr_dtype(lab)
    a.M = _ptr(M)
    a.src = _ptr(src)
    a.tgt = _ptr(tgt)
    a.step = _ptr(step)
    a.src_per_ray = 0 if src.shape[1] == 1 else 1
    a.B, a.N = B, N
    a.width = width
    a.n_samples = n_samples
    return a


def _set_M_lo(a: _ffi.RaymarchArgs, M_lo: torch.Tensor | None, M: torch.Tensor) -> None:
    """Point the arguments at the affine's low parts (kept alive by the caller)."""
    if M_lo is None or M_lo.numel() == 0:
        return
    if tuple(M_lo.shape) != tuple(M.shape) or M_lo.dtype != torch.float32 or not M_lo.is_contiguous():
        raise ValueError("M_lo must be a contiguous float32 tensor shaped like M")
    a.M_lo = M_lo.data_ptr()


def _apply_skip(a: _ffi.RaymarchArgs, skip, vol: torch.Tensor) -> None:
    """Fill the empty-space fields of the C-ABI arguments from an EmptySpace."""
    if skip is None or skip.mode == _ffi.NDRR_SKIP_NONE:
        return
    g = skip.grid
    if g.grid.device != vol.device or tuple(g.volume_shape) != tuple(vol.shape):
        raise ValueError("the occupancy grid was built for another volume or device")
    a.skip_mode = int(skip.mode)
    a.occ_cell = g.cell
    a.occ_gz, a.occ_gy, a.occ_gx = g.grid.shape
    a.occ_grid = g.grid.data_ptr()
    a.proposal_margin = float(skip.margin)
    if skip.mode == _ffi.NDRR_SKIP_PROPOSAL:
        a.proposal_params = skip.packed.data_ptr()


def skip_windows(
    vol: torch.Tensor,
    M: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    width: int,
    skip,
    stats: torch.Tensor | None = None,
    t_window: torch.Tensor | None = None,
) -> torch.Tensor:
    """Per-ray sample windows [B, N, 2] int32 (first sample, one past the
    last) of an `EmptySpace` skip, computed by their own kernel
    (ndrr_skip_windows); pass them to the march as `windows`."""
    _check_inputs(vol, vol, M, src, tgt, step, n_samples, 1)
    vol, _, M, src, tgt, step = _prep(vol, vol, M, src, tgt, step)
    B, N, _ = tgt.shape
    win = torch.empty(B, N, 2, device=vol.device, dtype=torch.int32)
    a = _base_args(vol, vol, M, src, tgt, step, n_samples, 1, width)
    _apply_skip(a, skip, vol)
    if t_window is not None:
        t_window = t_window.float().contiguous()
        a.t_window = _ptr(t_window)
    if stats is not None:
        if stats.dtype != torch.int64 or stats.numel() < 4 or not stats.is_contiguous():
            raise ValueError("stats must be a contiguous int64 tensor with 4 entries")
        a.skip_stats = stats.data_ptr()
    lib = _ffi.load()
    _ffi.check(lib.ndrr_skip_windows(ctypes.byref(a), _ptr(win), _stream_handle(vol.device)), "ndrr_skip_windows")
    return win


def _windows_route(skip) -> bool:
    """True when a skip is applied through per-ray windows: the learned
    proposal always, the occupancy skip when built with fused=False."""
    return skip is not None and (int(skip.mode) == _ffi.NDRR_SKIP_PROPOSAL or not getattr(skip, "fused", True))


def _check_windows(win: torch.Tensor, B: int, N: int) -> torch.Tensor:
    if win.dtype != torch.int32 or tuple(win.shape) != (B, N, 2):
        raise ValueError(f"windows must be an int32 [B, N, 2] = [{B}, {N}, 2] tensor")
    return win.contiguous()


def _prep(vol, lab, M, src, tgt, step):
    vol = vol.contiguous()
    lab = lab.contiguous()
    M = M.float().contiguous()
    src = src.float().contiguous()
    tgt = tgt.float().contiguous()
    step = step.float().contiguous()
    return vol, lab, M, src, tgt, step


def quad_volume(vol: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """Quad-layout copy of a [D, H, W] volume (see ndrr_quad_build): element
    (qz, qy, qx) holds the four x/y corners of a cell of plane qz - 2, with a
    zero border, so a trilinear sample is two vector loads. `out`: an earlier
    quad copy of a volume of the same shape and dtype, rebuilt in place."""
    if not vol.is_cuda or vol.dim() != 3 or vol.dtype not in _FLOAT_DTYPES:
        raise ValueError("quad_volume needs a [D, H, W] float CUDA tensor")
    vol = vol.contiguous()
    D, H, W = vol.shape
    es = 16 if vol.dtype == torch.float32 else 8
    nbytes = (D + 4) * (H + 3) * (W + 3) * es
    if out is not None:
        if out.dtype != torch.uint8 or out.numel() != nbytes or out.device != vol.device or not out.is_contiguous():
            raise ValueError("out is not a quad copy of a volume of this shape and dtype")
        q = out
    else:
        q = torch.empty(nbytes, device=vol.device, dtype=torch.uint8)
    lib = _ffi.load()
    _ffi.check(
        lib.ndrr_quad_build(vol.data_ptr(), ndrr_dtype(vol), D, H, W, q.data_ptr(), _stream_handle(vol.device)),
        "ndrr_quad_build",
    )
    return q


def quad_volume_labeled(vol: torch.Tensor, lab: torch.Tensor, n_classes: int,
                        out: torch.Tensor | None = None) -> torch.Tensor:
    """Labelled quad-layout copy of a 16-bit [D, H, W] volume and its label
    map (see ndrr_quad_build_labeled): 16 bytes per element, the quad's four
    corner values and the four corners' classes, so a per-label sample reads
    its nearest label from the two loads that bring its corners. Pass it as
    `quad` to the march (recognised by its size). n_classes in 2..255."""
    if not vol.is_cuda or vol.dim() != 3 or vol.dtype not in (torch.float16, torch.bfloat16):
        raise ValueError("quad_volume_labeled needs a [D, H, W] float16/bfloat16 CUDA tensor")
    if tuple(lab.shape) != tuple(vol.shape) or lab.device != vol.device:
        raise ValueError("the label map must match the volume's shape and device")
    if not 2 <= n_classes <= 255:
        raise ValueError("the labelled quad layout takes 2..255 classes")
    vol, lab = vol.contiguous(), lab.contiguous()
    D, H, W = vol.shape
    nbytes = (D + 4) * (H + 3) * (W + 3) * 16
    if out is not None:
        if out.dtype != torch.uint8 or out.numel() != nbytes or out.device != vol.device or not out.is_contiguous():
            raise ValueError("out is not a labelled quad copy of a volume of this shape")
        q = out
    else:
        q = torch.empty(nbytes, device=vol.device, dtype=torch.uint8)
    lib = _ffi.load()
    _ffi.check(
        lib.ndrr_quad_build_labeled(vol.data_ptr(), ndrr_dtype(vol), lab.data_ptr(), ndrr_dtype(lab), n_classes,
                                    D, H, W, q.data_ptr(), _stream_handle(vol.device)),
        "ndrr_quad_build_labeled",
    )
    return q


def quad_is_labeled(vol: torch.Tensor, quad: torch.Tensor) -> bool:
    """Whether `quad` is the labelled quad copy of `vol` (16 bytes per element
    for a 16-bit volume) rather than the plain one; any other size raises."""
    D, H, W = vol.shape
    n = (D + 4) * (H + 3) * (W + 3)
    es = quad.numel() // n if n else 0
    if quad.numel() != n * es or es not in ((16,) if vol.dtype == torch.float32 else (8, 16)):
        raise ValueError("quad is not a quad-layout copy of a volume of this shape and dtype")
    return vol.dtype != torch.float32 and es == 16


class TextureVolume:
    """Hardware-filtered 3-D texture of a float32 [D, H, W] volume
    (ndrr_texture_create) for the texture forward variant: pass it as
    `raymarch_forward(..., texture=...)`. Its trilinear weights have 8
    fractional bits, so results differ from the software path by about 1e-3
    relative; a measured variant, forward only. Frees its CUDA array on
    `close()` or when collected."""

    def __init__(self, vol: torch.Tensor):
        if not vol.is_cuda or vol.dim() != 3 or vol.dtype != torch.float32:
            raise ValueError("TextureVolume needs a float32 [D, H, W] CUDA tensor")
        vol = vol.contiguous()
        self.shape = tuple(vol.shape)
        self.device = vol.device
        h = ctypes.c_uint64(0)
        lib = _ffi.load()
        _ffi.check(lib.ndrr_texture_create(vol.data_ptr(), *self.shape, ctypes.byref(h), _stream_handle(vol.device)),
                   "ndrr_texture_create")
        self.handle = int(h.value)

    def close(self) -> None:
        if getattr(self, "handle", 0):
            torch.cuda.synchronize(self.device)
            _ffi.load().ndrr_texture_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass


def raymarch_forward(
    vol: torch.Tensor,
    lab: torch.Tensor,
    M: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    n_classes: int,
    width: int,
    t_window: torch.Tensor | None = None,
    with_total: bool = False,
    out_dtype: torch.dtype | None = None,
    tile: tuple[int, int, int] | None = None,
    skip=None,
    extent: torch.Tensor | None = None,
    stats: torch.Tensor | None = None,
    quad: torch.Tensor | None = None,
    windows: torch.Tensor | None = None,
    texture: TextureVolume | None = None,
    fwd_mode: int = 0,
    M_lo: torch.Tensor | None = None,
) -> tuple[torch.Tensor, torch.Tensor | None]:
    """Launch the forward kernel; returns (out [B, C, N], total [B, N] or None).

    `tile` optionally fixes the launch shape (tile_w, tile_h, sample_split).
    `skip` is an `EmptySpace` (empty-space skipping), `extent` an optional
    float32 [B, N, 2] output receiving each ray's non-empty interval in t,
    `stats` an optional int64 [4] counter tensor (see ndrr_raymarch_args),
    `quad` the volume's quad-layout copy (`quad_volume`), read instead of
    `vol` when given. The learned proposal, and an occupancy skip built with
    `fused=False`, are applied through per-ray windows (`skip_windows`);
    `windows` passes windows computed earlier. `M_lo` the low parts of the
    affine (M + M_lo; see ndrr_raymarch_args). `fwd_mode` 1 selects the
    TMA-staged forward (a measured variant: f32, one channel, no skipping)
    and `texture` the texture-filtered one (`TextureVolume`)."""
    _check_inputs(vol, lab, M, src, tgt, step, n_samples, n_classes)
    vol, lab, M, src, tgt, step = _prep(vol, lab, M, src, tgt, step)
    B, N, _ = tgt.shape
    if _windows_route(skip):
        if windows is None:
            windows = skip_windows(vol, M, src, tgt, step, n_samples, width, skip, stats=stats, t_window=t_window)
        skip, stats = None, None
    if windows is not None:
        windows = _check_windows(windows, B, N)
    odt = out_dtype or vol.dtype
    out = torch.empty(B, n_classes, N, device=vol.device, dtype=odt)
    total = torch.empty(B, N, device=vol.device, dtype=odt) if with_total else None
    a = _base_args(vol, lab, M, src, tgt, step, n_samples, n_classes, width)
    _set_M_lo(a, M_lo, M)
    a.out = _ptr(out)
    a.out_dtype = ndrr_dtype(out)
    a.out_total = _ptr(total)
    if t_window is not None:
        t_window = t_window.float().contiguous()
        if t_window.shape != (B, N, 2):
            raise ValueError(f"t_window must be [B, N, 2], got {tuple(t_window.shape)}")
        a.t_window = _ptr(t_window)
    if tile is not None:
        a.tile_w, a.tile_h, a.sample_split = (int(v) for v in tile)
    _apply_skip(a, skip, vol)
    if windows is not None:
        a.sample_window = _ptr(windows)
    if quad is not None and quad.numel():
        a.vol_quad = quad.data_ptr()
        a.quad_labels = int(quad_is_labeled(vol, quad))
    a.fwd_mode = int(fwd_mode)
    if texture is not None:
        if texture.shape != tuple(vol.shape) or texture.device != vol.device or not texture.handle:
            raise ValueError("the texture was made from another volume or device, or is closed")
        a.vol_texture = texture.handle
    if extent is not None:
        if extent.shape != (B, N, 2) or extent.dtype != torch.float32 or not extent.is_contiguous():
            raise ValueError("extent must be a contiguous float32 [B, N, 2] tensor")
        a.out_extent = extent.data_ptr()
    if stats is not None:
        if stats.dtype != torch.int64 or stats.numel() < 4 or not stats.is_contiguous():
            raise ValueError("stats must be a contiguous int64 tensor with 4 entries")
        a.skip_stats = stats.data_ptr()
    lib = _ffi.load()
    _ffi.check(lib.ndrr_raymarch_fwd(ctypes.byref(a), _stream_handle(vol.device)), "ndrr_raymarch_fwd")
    return out, total


def raymarch_backward(
    go: torch.Tensor,
    vol: torch.Tensor,
    lab: torch.Tensor,
    M: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    n_classes: int,
    width: int,
    need_gvol: bool,
    need_gcam: bool,
    t_window: torch.Tensor | None = None,
    gvol: torch.Tensor | None = None,
    gvol_mode: int = 0,
    brick_cap: int = 0,
    slab_mib: int = 0,
    tile: tuple[int, int, int] | None = None,
    skip=None,
    quad: torch.Tensor | None = None,
    windows: torch.Tensor | None = None,
    M_lo: torch.Tensor | None = None,
):
    """Launch the adjoint; returns (gvol, gM, gsrc, gtgt, gstep) in float32.

    `gvol`, when given, is a float32 [D, H, W] buffer the volume gradient is
    accumulated into (so several calls can share one); otherwise a zeroed one
    is allocated. `gvol_mode` selects the volume-gradient scatter (0 auto,
    1 direct atomics, 2 per-slab shared-memory brick, 3 slab-ordered work,
    which auto picks for the quad layout without camera gradients, 4 slab
    with warp aggregation, 5 split: a pose pass that gathers, then a
    slab-ordered scatter pass from sample positions alone),
    `slab_mib` the quad-gradient MiB per slab (0 = default), `brick_cap` the brick
    capacity in voxels (0 = default) and `tile` an explicit
    (tile_w, tile_h, sample_split) launch shape. Skips and `windows` apply to
    the pose/camera adjoint only: with `need_gvol` every sample is marched
    (gvol_mode 5 applies them to its pose pass)."""
    _check_inputs(vol, lab, M, src, tgt, step, n_samples, n_classes)
    vol, lab, M, src, tgt, step = _prep(vol, lab, M, src, tgt, step)
    B, N, _ = tgt.shape
    # With a volume gradient, sample windows reach the slab-ordered adjoint of
    # one channel (they spare the loads of zero-corner samples, all of which
    # are still scattered) and the split adjoint's pose pass; elsewhere every
    # sample is marched and the skip is dropped.
    quad_on = quad is not None and quad.numel() > 0
    slab_like = (gvol_mode in (_ffi.NDRR_GVOL_AUTO, _ffi.NDRR_GVOL_SLAB, _ffi.NDRR_GVOL_SLAB_WARP)
                 and quad_on and not need_gcam and n_classes == 1)
    if need_gvol and gvol_mode != _ffi.NDRR_GVOL_SPLIT and not (slab_like and windows is not None):
        skip, windows = None, None
    elif _windows_route(skip):
        if windows is None:
            windows = skip_windows(vol, M, src, tgt, step, n_samples, width, skip, t_window=t_window)
        skip = None
    if windows is not None:
        windows = _check_windows(windows, B, N)
    dev = vol.device
    go = go.contiguous()
    if go.shape != (B, n_classes, N):
        raise ValueError(f"go must be [B, C, N] = [{B}, {n_classes}, {N}], got {tuple(go.shape)}")
    if go.dtype not in _FLOAT_DTYPES:
        go = go.float()
    empty = torch.empty(0, device=dev, dtype=torch.float32)
    gM = torch.empty(B, 3, 4, device=dev, dtype=torch.float32)
    overwrite = False
    if need_gvol:
        if gvol is None:
            # with the quad layout the fold writes every voxel: no zeroing
            overwrite = quad_on
            gvol = (torch.empty if overwrite else torch.zeros)(vol.shape, device=dev, dtype=torch.float32)
        elif gvol.shape != vol.shape or gvol.dtype != torch.float32 or not gvol.is_contiguous():
            raise ValueError("gvol must be a contiguous float32 tensor shaped like the volume")
    else:
        gvol = empty
    if need_gcam:
        gsrc = torch.empty(src.shape, device=dev, dtype=torch.float32)
        gtgt = torch.empty(B, N, 3, device=dev, dtype=torch.float32)
        gstep = torch.empty(B, N, device=dev, dtype=torch.float32)
    else:
        gsrc = gtgt = gstep = empty
    a = _base_args(vol, lab, M, src, tgt, step, n_samples, n_classes, width)
    _set_M_lo(a, M_lo, M)
    a.go = _ptr(go)
    a.go_dtype = ndrr_dtype(go)
    a.need_gvol = int(need_gvol)
    a.need_gcam = int(need_gcam)
    a.gvol = _ptr(gvol) if need_gvol else None
    a.gM = _ptr(gM)
    if need_gcam:
        a.gsrc, a.gtgt, a.gstep = _ptr(gsrc), _ptr(gtgt), _ptr(gstep)
    if t_window is not None:
        t_window = t_window.float().contiguous()
        a.t_window = _ptr(t_window)
    a.gvol_mode = int(gvol_mode)
    a.brick_cap = int(brick_cap)
    a.slab_mib = int(slab_mib)
    _apply_skip(a, skip, vol)
    if windows is not None:
        a.sample_window = _ptr(windows)
    gq = None
    a.gvol_overwrite = int(overwrite)
    if quad_on:
        a.vol_quad = quad.data_ptr()
        a.quad_labels = int(quad_is_labeled(vol, quad))
        if need_gvol:
            D, H, W = vol.shape
            gq = torch.empty((D + 4) * (H + 3) * (W + 3) * 4, device=dev, dtype=torch.float32)
            a.gvol_quad = gq.data_ptr()
    if tile is not None:
        a.tile_w, a.tile_h, a.sample_split = (int(v) for v in tile)
    lib = _ffi.load()
    nbytes = ctypes.c_uint64(0)
    _ffi.check(lib.ndrr_raymarch_bwd_workspace_bytes(ctypes.byref(a), ctypes.byref(nbytes)), "workspace query")
    ws = torch.empty(max(int(nbytes.value), 16), device=dev, dtype=torch.uint8)
    a.workspace = ws.data_ptr()
    a.workspace_bytes = ws.numel()
    _ffi.check(lib.ndrr_raymarch_bwd(ctypes.byref(a), _stream_handle(dev)), "ndrr_raymarch_bwd")
    return gvol, gM, gsrc, gtgt, gstep


# --------------------------------------------------------------- custom ops
@torch.library.custom_op("nanodrr_gb300::fused_raymarch", mutates_args=())
def fused_raymarch(
    vol: torch.Tensor,
    lab: torch.Tensor,
    M: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    n_classes: int,
    width: int,
) -> torch.Tensor:
    """Differentiable ray march: [B, C, N] line integrals in `vol.dtype`."""
    out, _ = raymarch_forward(vol, lab, M, src, tgt, step, n_samples, n_classes, width)
    return out


@fused_raymarch.register_fake
def _(vol, lab, M, src, tgt, step, n_samples, n_classes, width):
    B, N, _ = tgt.shape
    return torch.empty(B, n_classes, N, device=vol.device, dtype=vol.dtype)


@torch.library.custom_op("nanodrr_gb300::fused_raymarch_bwd", mutates_args=())
def fused_raymarch_bwd(
    go: torch.Tensor,
    vol: torch.Tensor,
    lab: torch.Tensor,
    M: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    n_classes: int,
    width: int,
    need_gvol: bool,
    need_gcam: bool,
) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor]:
    """Adjoint launch; volume gradients use atomics (reference _fused.py:493-497)."""
    if need_gvol and torch.are_deterministic_algorithms_enabled():
        raise RuntimeError(
            "Volume gradients on the cuda backend use nondeterministic atomics; "
            "disable deterministic algorithms or detach the volume"
        )
    gvol, gM, gsrc, gtgt, gstep = raymarch_backward(
        go, vol, lab, M, src, tgt, step, n_samples, n_classes, width, need_gvol, need_gcam
    )
    return gvol, gM, gsrc, gtgt, gstep


@fused_raymarch_bwd.register_fake
def _(go, vol, lab, M, src, tgt, step, n_samples, n_classes, width, need_gvol, need_gcam):
    B, N, _ = tgt.shape
    gM = torch.empty(B, 3, 4, device=M.device, dtype=torch.float32)
    empty = gM.new_empty(0)
    gvol = torch.empty(vol.shape, device=M.device, dtype=torch.float32) if need_gvol else empty
    gsrc = torch.empty(src.shape, device=M.device, dtype=torch.float32) if need_gcam else empty
    gtgt = torch.empty(B, N, 3, device=M.device, dtype=torch.float32) if need_gcam else empty
    gstep = torch.empty(B, N, device=M.device, dtype=torch.float32) if need_gcam else empty
    return gvol, gM, gsrc, gtgt, gstep


def _setup_context(ctx, inputs, output):
    vol, lab, M, src, tgt, step, n_samples, n_classes, width = inputs
    ctx.save_for_backward(vol, lab, M.contiguous(), src, tgt, step)
    ctx.n_samples = n_samples
    ctx.n_classes = n_classes
    ctx.width = width


def _backward(ctx, go):
    vol, lab, M, src, tgt, step = ctx.saved_tensors
    need_gvol = ctx.needs_input_grad[0]
    need_gcam = any(ctx.needs_input_grad[i] for i in (3, 4, 5))
    gvol, gM, gsrc, gtgt, gstep = fused_raymarch_bwd(
        go, vol, lab, M, src, tgt, step, ctx.n_samples, ctx.n_classes, ctx.width, need_gvol, need_gcam
    )
    return (
        gvol.to(vol.dtype) if need_gvol else None,
        None,  # lab: nearest-label lookup, not differentiable
        gM.to(M.dtype),
        gsrc.to(src.dtype) if need_gcam else None,
        gtgt.to(tgt.dtype) if need_gcam else None,
        gstep.to(step.dtype) if need_gcam else None,
        None,
        None,
        None,
    )


torch.library.register_autograd("nanodrr_gb300::fused_raymarch", _backward, setup_context=_setup_context)


# ------------------------------------------------------- general op
# Same contract as fused_raymarch plus the layout and skip structures the
# render call uses: `quad` is the volume's quad-layout copy (or an empty
# tensor for the plain layout), `occ_grid`/`occ_cell`/`proposal`/`skip_mode`/
# `margin` the empty-space skipping (skip_mode 0 = none; see EmptySpace).
# Skipped samples have eight zero corners, so the output and the pose/camera
# gradients equal the plain march's; the volume gradient is computed over the
# full box-culled window.
class _SkipArgs:
    def __init__(self, grid, cell, packed, mode, margin, shape):
        from .empty_space import OccupancyGrid

        self.grid = OccupancyGrid(grid, cell, shape)
        self.packed = packed
        self.mode = mode
        self.margin = margin


def _skip_of(vol, occ_grid, occ_cell, proposal, skip_mode, margin):
    if skip_mode == 0:
        return None
    return _SkipArgs(occ_grid, occ_cell, proposal, skip_mode, margin, vol.shape)


@torch.library.custom_op("nanodrr_gb300::fused_raymarch_ex", mutates_args=())
def fused_raymarch_ex(
    vol: torch.Tensor,
    quad: torch.Tensor,
    lab: torch.Tensor,
    M: torch.Tensor,
    M_lo: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    n_classes: int,
    width: int,
    occ_grid: torch.Tensor,
    occ_cell: int,
    proposal: torch.Tensor,
    skip_mode: int,
    margin: float,
    windows_ahead: bool,
    slab_mib: int,
) -> tuple[torch.Tensor, torch.Tensor]:
    """Returns (out [B, C, N], windows): with `windows_ahead` and a skip, the
    per-ray sample windows [B, N, 2] int32 the forward used, which the
    pose/camera adjoint reuses; otherwise an empty int32 tensor. `slab_mib`
    is the adjoint's slab size (0 = default), passed through to it. `M_lo`
    holds the low parts of the affine (M + M_lo, see ndrr_raymarch_args) or
    is empty."""
    return fused_raymarch_ex_forward(vol, quad, lab, M, M_lo, src, tgt, step, n_samples, n_classes, width, occ_grid,
                                     occ_cell, proposal, skip_mode, margin, windows_ahead, slab_mib)


def fused_raymarch_ex_forward(vol, quad, lab, M, M_lo, src, tgt, step, n_samples, n_classes, width, occ_grid,
                              occ_cell, proposal, skip_mode, margin, windows_ahead, slab_mib):
    """The forward of `fused_raymarch_ex` without the op dispatch (the caller
    uses it when no gradient is recorded and nothing is being traced)."""
    skip = _skip_of(vol, occ_grid, occ_cell, proposal, skip_mode, margin)
    windows = None
    if skip is not None and (windows_ahead or _windows_route(skip)):
        windows = skip_windows(vol, M, src, tgt, step, n_samples, width, skip)
        skip = None
    out, _ = raymarch_forward(vol, lab, M, src, tgt, step, n_samples, n_classes, width, skip=skip, quad=quad,
                              windows=windows, M_lo=M_lo)
    if windows is None:
        windows = torch.empty(0, device=vol.device, dtype=torch.int32)
    return out, windows


@fused_raymarch_ex.register_fake
def _(vol, quad, lab, M, M_lo, src, tgt, step, n_samples, n_classes, width, occ_grid, occ_cell, proposal, skip_mode,
      margin, windows_ahead, slab_mib):
    B, N, _ = tgt.shape
    out = torch.empty(B, n_classes, N, device=vol.device, dtype=vol.dtype)
    ahead = skip_mode == _ffi.NDRR_SKIP_PROPOSAL or (skip_mode != 0 and windows_ahead)
    shape = (B, N, 2) if ahead else (0,)
    return out, torch.empty(shape, device=vol.device, dtype=torch.int32)


@torch.library.custom_op("nanodrr_gb300::fused_raymarch_ex_bwd", mutates_args=())
def fused_raymarch_ex_bwd(
    go: torch.Tensor,
    vol: torch.Tensor,
    quad: torch.Tensor,
    lab: torch.Tensor,
    M: torch.Tensor,
    M_lo: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    step: torch.Tensor,
    n_samples: int,
    n_classes: int,
    width: int,
    need_gvol: bool,
    need_gcam: bool,
    occ_grid: torch.Tensor,
    occ_cell: int,
    proposal: torch.Tensor,
    skip_mode: int,
    margin: float,
    windows: torch.Tensor,
    slab_mib: int,
) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor]:
    if need_gvol and torch.are_deterministic_algorithms_enabled():
        raise RuntimeError(
            "Volume gradients on the cuda backend use nondeterministic atomics; "
            "disable deterministic algorithms or detach the volume"
        )
    if windows.numel():
        skip, win = None, windows
    else:
        skip, win = _skip_of(vol, occ_grid, occ_cell, proposal, skip_mode, margin), None
    return raymarch_backward(
        go, vol, lab, M, src, tgt, step, n_samples, n_classes, width, need_gvol, need_gcam, skip=skip, quad=quad,
        windows=win, slab_mib=slab_mib, M_lo=M_lo,
    )


@fused_raymarch_ex_bwd.register_fake
def _(go, vol, quad, lab, M, M_lo, src, tgt, step, n_samples, n_classes, width, need_gvol, need_gcam, *rest):
    B, N, _ = tgt.shape
    gM = torch.empty(B, 3, 4, device=M.device, dtype=torch.float32)
    empty = gM.new_empty(0)
    gvol = torch.empty(vol.shape, device=M.device, dtype=torch.float32) if need_gvol else empty
    gsrc = torch.empty(src.shape, device=M.device, dtype=torch.float32) if need_gcam else empty
    gtgt = torch.empty(B, N, 3, device=M.device, dtype=torch.float32) if need_gcam else empty
    gstep = torch.empty(B, N, device=M.device, dtype=torch.float32) if need_gcam else empty
    return gvol, gM, gsrc, gtgt, gstep


def _ex_setup_context(ctx, inputs, output):
    (vol, quad, lab, M, M_lo, src, tgt, step, n_samples, n_classes, width, occ_grid, occ_cell, proposal, mode,
     margin, windows_ahead, slab_mib) = inputs
    ctx.save_for_backward(vol, quad, lab, M.contiguous(), M_lo, src, tgt, step, occ_grid, proposal, output[1])
    ctx.args = (n_samples, n_classes, width, occ_cell, mode, margin, slab_mib)


def _ex_backward(ctx, go, _gwin):
    vol, quad, lab, M, M_lo, src, tgt, step, occ_grid, proposal, windows = ctx.saved_tensors
    n_samples, n_classes, width, occ_cell, mode, margin, slab_mib = ctx.args
    need_gvol = ctx.needs_input_grad[0]
    need_gcam = any(ctx.needs_input_grad[i] for i in (5, 6, 7))
    gvol, gM, gsrc, gtgt, gstep = fused_raymarch_ex_bwd(
        go, vol, quad, lab, M, M_lo, src, tgt, step, n_samples, n_classes, width, need_gvol, need_gcam,
        occ_grid, occ_cell, proposal, mode, margin, windows, slab_mib,
    )
    return (
        gvol.to(vol.dtype) if need_gvol else None,
        None,  # quad: a derived copy of vol
        None,  # lab
        gM.to(M.dtype),
        None,  # M_lo: a rounding correction of M, not differentiated
        gsrc.to(src.dtype) if need_gcam else None,
        gtgt.to(tgt.dtype) if need_gcam else None,
        gstep.to(step.dtype) if need_gcam else None,
        None, None, None, None, None, None, None, None, None, None,
    )


torch.library.register_autograd("nanodrr_gb300::fused_raymarch_ex", _ex_backward, setup_context=_ex_setup_context)
