"""Intrinsics resample (2-D homography warp) — TEST INFRASTRUCTURE ONLY.

Restates the reference's `resample` (nanodrr src/nanodrr/camera/homography.py:
6-58) on CPU in torch: destination pixel p' = (x, y, 1) maps to the source
pixel p = K_old K_new^-1 p' (perspective divide), sampled bilinearly with
align_corners=True and zero padding, so p is in pixel units of the source
image (corners at integer pixel positions 0..W-1, 0..H-1). Autograd through
it is the reference's analytic backward.

`resample_pixels` is the same arithmetic written per corner (no
grid_sample), the form the CUDA kernel follows.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F


def resample_oracle(img: torch.Tensor, k_inv_old: torch.Tensor, k_inv_new: torch.Tensor) -> torch.Tensor:
    """[B, C, H, W] resampled images (homography.py:34-58)."""
    B, _, H, W = img.shape
    Hm = torch.linalg.inv(k_inv_old) @ k_inv_new
    ys, xs = torch.meshgrid(torch.arange(H, dtype=img.dtype), torch.arange(W, dtype=img.dtype), indexing="ij")
    coords = torch.stack([xs, ys, torch.ones_like(xs)], dim=-1).reshape(-1, 3).T
    src = (Hm @ coords).permute(0, 2, 1).reshape(B, H, W, 3)
    sx, sy = src[..., 0] / src[..., 2], src[..., 1] / src[..., 2]
    grid = torch.stack([sx / (W - 1) * 2 - 1, sy / (H - 1) * 2 - 1], dim=-1)
    return F.grid_sample(img, grid, align_corners=True, padding_mode="zeros", mode="bilinear")


def resample_pixels(img: torch.Tensor, Hm: torch.Tensor) -> torch.Tensor:
    """Per-corner bilinear form with the homography given directly [B, 3, 3]."""
    B, C, H, W = img.shape
    ys, xs = torch.meshgrid(torch.arange(H, dtype=img.dtype), torch.arange(W, dtype=img.dtype), indexing="ij")
    a = Hm[:, 0, 0, None, None] * xs + Hm[:, 0, 1, None, None] * ys + Hm[:, 0, 2, None, None]
    b = Hm[:, 1, 0, None, None] * xs + Hm[:, 1, 1, None, None] * ys + Hm[:, 1, 2, None, None]
    c = Hm[:, 2, 0, None, None] * xs + Hm[:, 2, 1, None, None] * ys + Hm[:, 2, 2, None, None]
    sx, sy = a / c, b / c
    x0, y0 = torch.floor(sx), torch.floor(sy)
    fx, fy = sx - x0, sy - y0
    out = torch.zeros_like(img)
    flat = img.reshape(B, C, H * W)
    for dy, wy in ((0, 1 - fy), (1, fy)):
        for dx, wx in ((0, 1 - fx), (1, fx)):
            xi, yi = x0 + dx, y0 + dy
            ok = (xi >= 0) & (xi <= W - 1) & (yi >= 0) & (yi <= H - 1)
            idx = (yi.clamp(0, H - 1) * W + xi.clamp(0, W - 1)).long().reshape(B, 1, H * W).expand(B, C, H * W)
            v = torch.gather(flat, 2, idx).reshape(B, C, H, W)
            out = out + torch.where(ok[:, None], v * (wx * wy)[:, None], torch.zeros_like(v))
    return out
