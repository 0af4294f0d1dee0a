"""Intrinsics resample: `resample(img, k_inv_old, k_inv_new)`.

Same call and result as the reference's `resample` (nanodrr
src/nanodrr/camera/homography.py:6-58): each destination pixel p' maps to the
source pixel p = K_old K_new^-1 p' and is sampled bilinearly (align_corners,
zero padding). The warp and its adjoint run in the library
(`ndrr_homography_resample{,_bwd}`); the 3x3 homography and its chain to the
two inverse intrinsics are tiny torch expressions (an explicit cofactor
inverse, no linear-algebra library). Differentiable in the image and both
intrinsics. Float32 images on CUDA.
"""

from __future__ import annotations

import ctypes

import torch

from . import _ffi
from .geometry import mm_small


def _inv3(A: torch.Tensor) -> torch.Tensor:
    """Inverse of [..., 3, 3] matrices by cofactors (differentiable)."""
    a, b, c = A[..., 0, 0], A[..., 0, 1], A[..., 0, 2]
    d, e, f = A[..., 1, 0], A[..., 1, 1], A[..., 1, 2]
    g, h, i = A[..., 2, 0], A[..., 2, 1], A[..., 2, 2]
    co = torch.stack([
        e * i - f * h, c * h - b * i, b * f - c * e,
        f * g - d * i, a * i - c * g, c * d - a * f,
        d * h - e * g, b * g - a * h, a * e - b * d,
    ], dim=-1).reshape(A.shape)
    det = a * co[..., 0, 0] + b * co[..., 1, 0] + c * co[..., 2, 0]
    return co / det[..., None, None]


def _stream(dev) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _check(img: torch.Tensor, hom: torch.Tensor):
    if not img.is_cuda:
        raise RuntimeError("nanodrr_gb300 resamples on CUDA devices only (got an image on %s)" % img.device)
    if img.dim() != 4:
        raise ValueError(f"img must be [B, C, H, W], got {tuple(img.shape)}")
    if img.dtype != torch.float32:
        raise ValueError(f"img dtype {img.dtype} unsupported; the CUDA resample takes float32")
    B = img.shape[0]
    if hom.shape != (B, 3, 3):
        raise ValueError(f"homography must be [B, 3, 3] = [{B}, 3, 3], got {tuple(hom.shape)}")


@torch.library.custom_op("nanodrr_gb300::homography_resample", mutates_args=())
def homography_resample(img: torch.Tensor, hom: torch.Tensor) -> torch.Tensor:
    """[B, C, H, W] warp of `img` by the destination -> source homography."""
    _check(img, hom)
    img = img.contiguous()
    hom = hom.float().contiguous()
    B, C, H, W = img.shape
    out = torch.empty_like(img)
    lib = _ffi.load()
    _ffi.check(lib.ndrr_homography_resample(img.data_ptr(), hom.data_ptr(), B, C, H, W, out.data_ptr(),
                                            _stream(img.device)), "ndrr_homography_resample")
    return out


@homography_resample.register_fake
def _(img, hom):
    return torch.empty_like(img)


@torch.library.custom_op("nanodrr_gb300::homography_resample_bwd", mutates_args=())
def homography_resample_bwd(go: torch.Tensor, img: torch.Tensor, hom: torch.Tensor, need_gimg: bool,
                            need_ghom: bool) -> tuple[torch.Tensor, torch.Tensor]:
    img = img.contiguous()
    hom = hom.float().contiguous()
    go = go.float().contiguous()
    B, C, H, W = img.shape
    gimg = torch.zeros_like(img) if need_gimg else img.new_empty(0)
    ghom = torch.empty(B, 3, 3, device=img.device) if need_ghom else img.new_empty(0)
    lib = _ffi.load()
    nb = ctypes.c_uint64(0)
    _ffi.check(lib.ndrr_homography_resample_bwd_workspace_bytes(B, H, W, ctypes.byref(nb)), "workspace")
    ws = torch.empty(max(int(nb.value), 16), device=img.device, dtype=torch.uint8)
    _ffi.check(lib.ndrr_homography_resample_bwd(
        go.data_ptr(), img.data_ptr(), hom.data_ptr(), B, C, H, W,
        gimg.data_ptr() if need_gimg else None, ghom.data_ptr() if need_ghom else None,
        ws.data_ptr(), ws.numel(), _stream(img.device)), "ndrr_homography_resample_bwd")
    return gimg, ghom


@homography_resample_bwd.register_fake
def _(go, img, hom, need_gimg, need_ghom):
    B = img.shape[0]
    return (torch.empty_like(img) if need_gimg else img.new_empty(0),
            img.new_empty(B, 3, 3) if need_ghom else img.new_empty(0))


def _setup(ctx, inputs, output):
    img, hom = inputs
    ctx.save_for_backward(img, hom)


def _backward(ctx, go):
    img, hom = ctx.saved_tensors
    need_gimg, need_ghom = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
    gimg, ghom = homography_resample_bwd(go, img, hom, need_gimg, need_ghom)
    return (gimg if need_gimg else None, ghom.to(hom.dtype) if need_ghom else None)


torch.library.register_autograd("nanodrr_gb300::homography_resample", _backward, setup_context=_setup)


def resample(img: torch.Tensor, k_inv_old: torch.Tensor, k_inv_new: torch.Tensor) -> torch.Tensor:
    """Resample images from one camera's inverse intrinsics to another's
    (reference homography.py:6-58): H = K_old K_new^-1 = inv(k_inv_old) @
    k_inv_new, applied to destination pixel coordinates."""
    hom = mm_small(_inv3(k_inv_old.float()), k_inv_new.float())
    if hom.shape[0] != img.shape[0]:
        hom = hom.expand(img.shape[0], 3, 3)
    return homography_resample(img, hom.contiguous())
