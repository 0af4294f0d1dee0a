"""Normalised cross-correlation — TEST INFRASTRUCTURE ONLY.

Restates the reference's NormalizedCrossCorrelation2d (nanodrr
src/nanodrr/metrics/ncc.py:8-37, patch unfolding :65-74) in torch on CPU in
any dtype: per channel (or per p x p window unfolded into channels) both
images are centred and divided by sqrt(population variance + eps); the score
is the mean of the products over channels and pixels.
"""

from __future__ import annotations

import torch


def _norm(x: torch.Tensor, eps: float) -> torch.Tensor:
    mu = x.mean(dim=(-1, -2), keepdim=True)
    var = x.var(dim=(-1, -2), keepdim=True, correction=0) + eps
    return (x - mu) / var.sqrt()


def _patches(x: torch.Tensor, p: int) -> torch.Tensor:
    x = x.unfold(2, p, step=1).unfold(3, p, step=1).contiguous()
    b, c, h, w, p1, p2 = x.shape
    return x.reshape(b, c * h * w, p1, p2)


def ncc_oracle(x1: torch.Tensor, x2: torch.Tensor, patch_size: int | None = None, eps: float = 1e-7) -> torch.Tensor:
    """Score [B] of two [B, C, H, W] batches (ncc.py:18-37)."""
    if patch_size is not None:
        x1, x2 = _patches(x1, patch_size), _patches(x2, patch_size)
    _, c, h, w = x1.shape
    return (_norm(x1, eps) * _norm(x2, eps)).sum(dim=(1, 2, 3)) / (c * h * w)
