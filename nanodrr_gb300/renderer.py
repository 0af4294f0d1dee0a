"""`render`: the user-facing call, a drop-in for the reference's fused backend.

Mirrors nanodrr's `render` (src/nanodrr/drr/renderer.py:21-98) and the
adapter `render_fused` (src/nanodrr/drr/backends.py:72-117): same arguments,
same ray construction (`_make_tgt`/`_make_src`, renderer.py:101-132), same
camera-space step size (renderer.py:82) and the same camera -> voxel affine
`M = (world_to_voxel @ rt_inv)[:, :3]` in float32 (backends.py:96). There is
one backend, the sm_103a CUDA kernels: `backend` accepts "auto", "cuda" and
"triton" (the reference's name for its fused backend, kept so existing calls
switch unchanged); any other value raises, and CPU tensors raise rather than
falling back to a CPU path.
"""

from __future__ import annotations

import weakref

import torch

from . import _ffi
from .raymarch import (
    fused_raymarch_ex,
    fused_raymarch_ex_forward,
    quad_volume,
    quad_volume_labeled,
)
from .subject import Subject

_BACKENDS = ("auto", "cuda", "triton")

# Ray set-ups (src, tgt, step expanded to the batch) of recent render calls,
# keyed by the intrinsics and sdd tensor objects: a repeated render with the
# same camera reuses them instead of rebuilding N rays with a dozen small
# launches. An entry is valid while both tensors are alive (weak references)
# and unmodified (version counters).
_RAY_CACHE: dict = {}
_RAY_CACHE_SIZE = 4

# Camera -> voxel affines of recent calls without a gradient, keyed by the
# world_to_voxel and rt_inv tensor objects: a repeated render of the same
# pose reuses M instead of two tensor launches (~25 us of host time per call).
# Valid while both tensors are alive and unmodified, as for the ray cache.
_M_CACHE: dict = {}
_M_CACHE_SIZE = 4


def fused_supported(subject: Subject, B: int, n_pixels: int) -> bool:
    """Limits of the CUDA kernels: one volume, int32 voxel and ray indexing
    (reference backends.py:66-69)."""
    N = B * n_pixels
    return subject.image.shape[0] == 1 and max(subject.image.numel(), subject.n_classes * N, 3 * N) < 2**31


def _make_tgt(k_inv, sdd, height, width, device, dtype) -> torch.Tensor:
    """Detector pixel centres (u + 0.5, v + 0.5, 1) mapped by sdd * K^-1."""
    N = height * width
    v, u = torch.meshgrid(
        torch.arange(height, device=device, dtype=dtype) + 0.5,
        torch.arange(width, device=device, dtype=dtype) + 0.5,
        indexing="ij",
    )
    uv1 = torch.stack([u, v, torch.ones_like(u)], dim=-1).reshape(N, 3)
    # K^-1 @ uv1 as three broadcast multiply-adds: no library GEMM for a 3x3
    # product, so the call also runs under torch's deterministic mode.
    k = k_inv[:, None]  # [B, 1, 3, 3]
    rays = k[..., 0] * uv1[None, :, 0:1] + k[..., 1] * uv1[None, :, 1:2] + k[..., 2] * uv1[None, :, 2:3]
    return sdd[:, None, None] * rays


def _make_src(orthographic: bool, tgt: torch.Tensor, sdd: torch.Tensor) -> torch.Tensor:
    """Point source at the camera origin, or parallel rays for orthographic."""
    if orthographic:
        src = tgt.clone()
        src[..., 2] -= sdd[:, None]
        return src
    B = tgt.shape[0]
    return torch.zeros(B, 1, 3, device=tgt.device, dtype=tgt.dtype)


def _camera_rays(k_inv, sdd, height, width, orthographic, device, dtype) -> tuple[torch.Tensor, torch.Tensor]:
    """(src, tgt) of the detector. Float32 CUDA cameras that need no gradient
    take one `ndrr_camera_rays` launch, which rounds every product and sum as
    `_make_tgt`/`_make_src` do, so the rays are bitwise the same; other
    cameras (a differentiable K^-1 or sdd, float64, traced calls) use the
    tensor expressions."""
    compiling = hasattr(torch, "compiler") and torch.compiler.is_compiling()
    want = torch.device(device)
    if (
        not compiling
        and dtype == torch.float32
        and k_inv.dtype == torch.float32
        and sdd.dtype == torch.float32
        and k_inv.is_cuda
        and k_inv.device == sdd.device
        and want.type == "cuda"
        and (want.index is None or want == k_inv.device)
        and k_inv.dim() == 3
        and tuple(k_inv.shape[1:]) == (3, 3)
        and sdd.dim() == 1
        and not (torch.is_grad_enabled() and (k_inv.requires_grad or sdd.requires_grad))
    ):
        n_k, n_s = k_inv.shape[0], sdd.shape[0]
        B = max(n_k, n_s)
        if n_k in (1, B) and n_s in (1, B):
            k = k_inv.detach().contiguous()
            s = sdd.detach().contiguous()
            N = height * width
            tgt = torch.empty(B, N, 3, device=k.device, dtype=torch.float32)
            src = torch.empty(B, N if orthographic else 1, 3, device=k.device, dtype=torch.float32)
            lib = _ffi.load()
            _ffi.check(
                lib.ndrr_camera_rays(k.data_ptr(), n_k, s.data_ptr(), n_s, B, height, width, int(bool(orthographic)),
                                     src.data_ptr(), tgt.data_ptr(), torch.cuda.current_stream(k.device).cuda_stream),
                "ndrr_camera_rays",
            )
            return src, tgt
    tgt = _make_tgt(k_inv, sdd, height, width, device, dtype)
    return _make_src(orthographic, tgt, sdd), tgt


def _affine_product(A3: torch.Tensor, rt: torch.Tensor) -> torch.Tensor:
    """(A @ rt)[:, :3, :] for A3 = A[:3] ([3, 4]) and rt [B, 4, 4], written as a
    broadcast sum (camera -> voxel affine of the reference, backends.py:96)."""
    return (A3[None, :, :, None] * rt[:, None, :, :]).sum(dim=2)


def _call_affine(w2v: torch.Tensor, rt_inv: torch.Tensor, grad: bool) -> torch.Tensor:
    """M = (world_to_voxel @ rt_inv)[:, :3] in float32 (`_affine_product`),
    from the affine cache when no gradient is recorded and nothing is traced
    or captured into a CUDA graph (a graph must read rt_inv on every replay)."""
    if (grad or (hasattr(torch, "compiler") and torch.compiler.is_compiling())
            or rt_inv.device.type != "cuda" or torch.cuda.is_current_stream_capturing()):
        return _affine_product(w2v.float()[:3], rt_inv.float())
    stream = torch.cuda.current_stream(rt_inv.device)
    key = (id(w2v), id(rt_inv))
    hit = _M_CACHE.get(key)
    if hit is not None:
        wref, wver, rref, rver, M, made_on = hit
        if wref() is w2v and rref() is rt_inv and wver == w2v._version and rver == rt_inv._version:
            if stream != made_on:  # keep the allocator from reusing it under this stream's kernels
                M.record_stream(stream)
            return M
    M = _affine_product(w2v.float()[:3], rt_inv.float())
    for k in [k for k, v in _M_CACHE.items() if v[0]() is None or v[2]() is None]:
        del _M_CACHE[k]  # entries whose tensors are gone
    while len(_M_CACHE) >= _M_CACHE_SIZE:
        _M_CACHE.pop(next(iter(_M_CACHE)))
    _M_CACHE[key] = (weakref.ref(w2v), w2v._version, weakref.ref(rt_inv), rt_inv._version, M, stream)
    return M


def compact_label(subject: Subject) -> torch.Tensor:
    """Label map for the kernels: float labels with n_classes <= 255 are packed
    to uint8 once per label tensor version (trunc(label) if it is a class in
    [0, C), else 255, which the kernels drop), saving 3 of 4 bytes per label
    read with identical routing. Other label maps pass through unchanged."""
    lab = subject.label[0, 0]
    C = subject.n_classes
    if not lab.is_floating_point() or C > 255:
        return lab.contiguous()
    key = (lab.data_ptr(), lab._version, lab.dtype, tuple(lab.shape), C, lab.device)
    cache = getattr(subject, "_ndrr_label_cache", None)
    if cache is not None and cache[0] == key:
        return cache[1]
    t = torch.trunc(lab.float())
    packed = torch.where((t >= 0) & (t < C), t, torch.full_like(t, 255.0)).to(torch.uint8).contiguous()
    object.__setattr__(subject, "_ndrr_label_cache", (key, packed))
    return packed


def render_cuda(subject, rt_inv, src, tgt, step_size, n_samples, height, width) -> torch.Tensor:
    """Adapter from the render call to the `nanodrr_gb300::fused_raymarch_ex` op (the
    reference's `fused_raymarch` contract plus the layout, skip and the
    affine's low parts)."""
    C = subject.n_classes
    img = subject.image
    # A reshape of the [1, 1, D, H, W] image back-propagates as a view; an
    # index ([0, 0]) would allocate and zero a volume-sized gradient per level.
    vol = (img.reshape(img.shape[-3:]) if img.shape[:2] == (1, 1) else img[0, 0]).contiguous()
    lab = compact_label(subject) if C > 1 else vol
    # With a gradient recorded, the adjoint forms sample positions from M +
    # M_lo in float-float and carries them in fixed point
    # (ndrr_raymarch_args.M_lo): M_lo is the float32 product's error against
    # the float64 affine of the same inputs. The forward reads float32 M only,
    # so a call without a gradient skips the float64 product.
    grad = torch.is_grad_enabled() and any(t.requires_grad for t in (vol, rt_inv, src, tgt, step_size))
    M = _call_affine(subject.world_to_voxel, rt_inv, grad)
    if grad:
        M64 = _affine_product(subject.world_to_voxel.detach().double()[:3], rt_inv.detach().double())
        M_lo = (M64 - M.detach().double()).float()
    else:
        M_lo = M.new_empty(0)
    B = max(M.shape[0], tgt.shape[0])
    if M.shape[0] != B:
        M = M.expand(B, -1, -1)
        if grad:
            M_lo = M_lo.expand(B, -1, -1)
    if not fused_supported(subject, B, height * width):
        raise ValueError("inputs exceed the CUDA kernel's limits (int32 indexing)")
    args = (
        vol,
        lab,
        M.contiguous(),
        src.expand(B, -1, -1).float().contiguous(),
        tgt.expand(B, -1, -1).float().contiguous(),
        step_size.expand(B, -1).float().contiguous(),
        n_samples,
        C,
        width,
    )
    skip = getattr(subject, "empty_space", None)
    # The quad copy is cached by the volume's address and version, which a
    # traced graph cannot read: under torch.compile the plain layout is used.
    compiling = hasattr(torch, "compiler") and torch.compiler.is_compiling()
    if skip is not None and not compiling:
        skip.grid.refresh(vol)  # the grid must describe the volume rendered
    # The quad copy (4x the volume's bytes) pays when many poses reuse it
    # through L2; one pose streams it once, and a one-pose forward read 408 MB
    # from DRAM in 73.6 us (82 % of HBM) where the plain volume took 52 us
    # (512 x 512 x 400 f32, 200^2 x 500 samples). A forward of one pose with no
    # gradient recorded therefore reads the plain volume; same image either way.
    default = "plain" if (not grad and B == 1) else "quad"
    layout = "plain" if compiling else (getattr(subject, "layout", None) or default)
    # Without a recorded gradient the forward is called directly, skipping
    # the custom op's dispatch (tens of microseconds of host time per call).
    direct = not compiling and not grad
    quad = cached_quad(subject, vol, lab, C) if layout == "quad" else vol.new_empty(0, dtype=torch.uint8)
    empty = vol.new_empty(0, dtype=torch.uint8)
    if skip is not None:
        # With a gradient recorded the skip always goes through sample windows
        # computed ahead of the march (not the in-kernel walk of a fused
        # occupancy skip): the adjoint reuses them, and with a volume gradient
        # they spare the loads of zero-corner samples (every sample is still
        # scattered).
        sk = (skip.grid.grid, skip.grid.cell, skip.packed, int(skip.mode), float(skip.margin),
              (not getattr(skip, "fused", True)) or grad)
    else:
        sk = (empty, 0, empty, 0, 0.0, False)
    slab_mib = int(getattr(subject, "slab_mib", 0))
    op = fused_raymarch_ex_forward if direct else fused_raymarch_ex
    out = op(args[0], quad, args[1], args[2], M_lo.contiguous(), *args[3:], *sk, slab_mib)[0]
    return out.reshape(B, C, height, width)


def labeled_quad_applies(vol: torch.Tensor, n_classes: int) -> bool:
    """Per-label renders of 16-bit volumes read the labelled quad layout:
    the class of a sample rides in the loads of its corners."""
    return vol.dtype in (torch.float16, torch.bfloat16) and 2 <= n_classes <= 255


def quad_cache_key(vol: torch.Tensor, lab: torch.Tensor | None, n_classes: int) -> tuple:
    key = (vol.data_ptr(), vol._version, vol.dtype, tuple(vol.shape), vol.device)
    if lab is not None and labeled_quad_applies(vol, n_classes):
        key += (lab.data_ptr(), lab._version, lab.dtype, n_classes)
    return key


def build_quad(vol: torch.Tensor, lab: torch.Tensor | None, n_classes: int, out: torch.Tensor | None = None):
    if lab is not None and labeled_quad_applies(vol, n_classes):
        return quad_volume_labeled(vol.detach(), lab, n_classes, out=out)
    return quad_volume(vol.detach(), out=out)


def cached_quad(subject, vol: torch.Tensor, lab: torch.Tensor | None = None, n_classes: int = 1) -> torch.Tensor:
    """The volume's quad-layout copy (labelled with `lab`'s classes for a
    per-label render of a 16-bit volume), rebuilt whenever the volume or
    label tensor or their contents (version counters) change."""
    key = quad_cache_key(vol, lab, n_classes)
    cache = getattr(subject, "_ndrr_quad_cache", None)
    if cache is not None and cache[0] == key:
        return cache[1]
    q = build_quad(vol, lab, n_classes)
    object.__setattr__(subject, "_ndrr_quad_cache", (key, q, lab, n_classes))
    return q


def render(
    subject: Subject,
    k_inv: torch.Tensor,
    rt_inv: torch.Tensor,
    sdd: torch.Tensor,
    height: int,
    width: int,
    n_samples: int = 500,
    orthographic: bool = False,
    src: torch.Tensor | None = None,
    tgt: torch.Tensor | None = None,
    backend: str = "auto",
) -> torch.Tensor:
    """Differentiable DRR: [B, C, H, W] line integrals of `subject.image`
    (per label channel when the subject has a multi-class label map).

    Args mirror the reference: `k_inv` [B|1, 3, 3], `rt_inv` [B, 4, 4]
    (camera -> world), `sdd` [B|1]; optional precomputed camera-space ray
    endpoints `src` [B, 1|N, 3] and `tgt` [B, N, 3]. Gradients flow to the
    pose, the intrinsics, the ray endpoints and the volume."""
    if n_samples < 2:
        raise ValueError("n_samples must be at least 2")
    if backend not in _BACKENDS:
        raise ValueError(f"Unknown backend {backend!r}; expected 'auto', 'cuda', or 'triton'")
    if not rt_inv.is_cuda or not subject.image.is_cuda:
        raise RuntimeError("nanodrr_gb300 renders on CUDA devices only; move the subject and poses to a GPU")
    device, dtype = rt_inv.device, rt_inv.dtype
    if tgt is None and src is None:
        rays = _cached_rays(k_inv, sdd, height, width, n_samples, orthographic, rt_inv)
        if rays is not None:
            return render_cuda(subject, rt_inv, *rays, n_samples, height, width)
    if tgt is None and src is None:
        src, tgt = _camera_rays(k_inv, sdd, height, width, orthographic, device, dtype)
    if tgt is None:
        tgt = _make_tgt(k_inv, sdd, height, width, device, dtype)
    if src is None:
        src = _make_src(orthographic, tgt, sdd)
    step_size = (tgt - src).norm(dim=-1) / float(n_samples - 1)
    return render_cuda(subject, rt_inv, src, tgt, step_size, n_samples, height, width)


def _cached_rays(k_inv, sdd, height, width, n_samples, orthographic, rt_inv):
    """(src, tgt, step) of the render call, float32, expanded to the batch and
    contiguous, from the ray cache or built and stored there; None when the
    call differentiates the camera (k_inv or sdd requires a gradient), is
    traced, or is captured into a CUDA graph (a graph must own its rays: a
    cache entry may be evicted and freed while the graph still replays)."""
    if k_inv.requires_grad or sdd.requires_grad:
        return None
    if hasattr(torch, "compiler") and torch.compiler.is_compiling():
        return None
    device, dtype = rt_inv.device, rt_inv.dtype
    if device.type != "cuda" or torch.cuda.is_current_stream_capturing():
        return None
    stream = torch.cuda.current_stream(device)
    B = max(rt_inv.shape[0], k_inv.shape[0], sdd.shape[0])
    key = (id(k_inv), id(sdd), height, width, n_samples, bool(orthographic), B, dtype, device)
    hit = _RAY_CACHE.get(key)
    if hit is not None:
        kref, kver, sref, sver, rays, made_on = hit
        if kref() is k_inv and sref() is sdd and kver == k_inv._version and sver == sdd._version:
            if stream != made_on:  # keep the allocator from reusing them under this stream's kernels
                for t in rays:
                    t.record_stream(stream)
            return rays
    src, tgt = _camera_rays(k_inv, sdd, height, width, orthographic, device, dtype)
    step = (tgt - src).norm(dim=-1) / float(n_samples - 1)
    rays = (src.expand(B, -1, -1).float().contiguous(), tgt.expand(B, -1, -1).float().contiguous(),
            step.expand(B, -1).float().contiguous())
    for k in [k for k, v in _RAY_CACHE.items() if v[0]() is None or v[2]() is None]:
        del _RAY_CACHE[k]  # entries whose camera tensors are gone
    while len(_RAY_CACHE) >= _RAY_CACHE_SIZE:
        _RAY_CACHE.pop(next(iter(_RAY_CACHE)))
    _RAY_CACHE[key] = (weakref.ref(k_inv), k_inv._version, weakref.ref(sdd), sdd._version, rays, stream)
    return rays
