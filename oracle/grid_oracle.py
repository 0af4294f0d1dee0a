"""Restatement of the reference's `render_torch` on CPU (test infrastructure).

Follows nanodrr src/nanodrr/drr/backends.py:9-63 step by step, with the ray
construction of src/nanodrr/drr/renderer.py:82, 101-132 and the grid affine
of src/nanodrr/data/subject.py:218-242. Inputs are plain tensors instead of a
Subject so that any dtype (float64 included) can be used throughout.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F


def voxel_to_grid(shape, dtype=torch.float64) -> torch.Tensor:
    """subject.py:218-242: voxel index i -> (2 i + 1) / S - 1 per axis."""
    D, H, W = shape[-3:]
    size = torch.tensor([W, H, D], dtype=dtype)
    mat = torch.eye(4, dtype=dtype)
    mat[:3, :3] = torch.diag(2.0 / size)
    mat[:3, 3] = 1.0 / size - 1.0
    return mat


def transform_point(xform: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """geometry/transform.py:15-28."""
    h = torch.einsum("b...ij,b...j->b...i", xform, torch.cat([v, torch.ones_like(v[..., :1])], dim=-1))
    return h[..., :-1] / h[..., -1:]


def make_tgt(k_inv, sdd, height, width, dtype=torch.float64) -> torch.Tensor:
    """renderer.py:101-117."""
    v, u = torch.meshgrid(
        torch.arange(height, dtype=dtype) + 0.5, torch.arange(width, dtype=dtype) + 0.5, indexing="ij"
    )
    uv1 = torch.stack([u, v, torch.ones_like(u)], dim=-1).reshape(height * width, 3)
    return sdd.to(dtype)[:, None, None] * torch.einsum("bij,nj->bni", k_inv.to(dtype), uv1)


def make_src(orthographic: bool, tgt: torch.Tensor, sdd: torch.Tensor) -> torch.Tensor:
    """renderer.py:120-132."""
    if orthographic:
        src = tgt.clone()
        src[..., 2] -= sdd.to(tgt.dtype)[:, None]
        return src
    return torch.zeros(tgt.shape[0], 1, 3, dtype=tgt.dtype)


def render_oracle(
    image: torch.Tensor,
    label: torch.Tensor | None,
    world_to_voxel: torch.Tensor,
    rt_inv: torch.Tensor,
    src: torch.Tensor,
    tgt: torch.Tensor,
    n_samples: int,
    n_classes: int = 1,
    step_size: torch.Tensor | None = None,
    drop_out_of_range: bool = True,
) -> torch.Tensor:
    """[B, C, N] DRR by grid_sample, all in image.dtype (backends.py:26-63).

    `image` and `label` are [D, H, W]; `world_to_voxel` [4, 4]; `rt_inv`
    [B, 4, 4]; `src` [B, 1|N, 3]; `tgt` [B, N, 3]. step_size defaults to
    |tgt - src| / (n - 1) (renderer.py:82). Labels outside [0, C) are dropped
    when `drop_out_of_range` (the fused kernel's rule, _fused.py:300); the
    reference's scatter_add_ would index out of bounds on them instead."""
    dt = image.dtype
    B = max(rt_inv.shape[0], tgt.shape[0])
    src = src.to(dt).expand(B, -1, -1)
    tgt = tgt.to(dt).expand(B, -1, -1)
    if step_size is None:
        step_size = (tgt - src).norm(dim=-1) / float(n_samples - 1)
    step_size = step_size.to(dt).expand(B, -1)
    N = tgt.shape[1]
    world_to_grid = voxel_to_grid(image.shape, dt) @ world_to_voxel.to(dt)
    xform = world_to_grid @ rt_inv.to(dt)
    xform = xform.expand(B, -1, -1)
    s = transform_point(xform, src)
    t_ = transform_point(xform, tgt)
    t = torch.linspace(0, 1, n_samples, dtype=dt)
    pts = torch.lerp(s[:, None, :, None], t_[:, None, :, None], t[None, :, None, None, None])
    img = F.grid_sample(image[None, None].expand(B, -1, -1, -1, -1), pts, mode="bilinear", align_corners=False)[
        :, 0, ..., 0
    ]  # [B, n, N]
    if n_classes == 1:
        return img.sum(dim=1, keepdim=True) * step_size[:, None, :]
    idx = F.grid_sample(
        label.to(dt)[None, None].expand(B, -1, -1, -1, -1), pts, mode="nearest", align_corners=False
    )[:, 0, ..., 0].long()
    if drop_out_of_range:
        keep = (idx >= 0) & (idx < n_classes)
        img = img * keep.to(dt)
        idx = torch.where(keep, idx, torch.zeros_like(idx))
    out = torch.zeros(B, n_classes, N, dtype=dt)
    out = out.scatter_add(1, idx, img)
    return out * step_size[:, None, :]


def render_oracle_chunked(image, label, world_to_voxel, rt_inv, src, tgt, n_samples, n_classes=1, chunk=4096):
    """`render_oracle` over ray chunks (bounded memory), no autograd."""
    B, N, _ = tgt.shape
    outs = []
    with torch.no_grad():
        for b in range(B):
            parts = []
            for i in range(0, N, chunk):
                s = src[b : b + 1, i : i + chunk] if src.shape[1] == N else src[b : b + 1]
                parts.append(
                    render_oracle(
                        image, label, world_to_voxel, rt_inv[b : b + 1], s, tgt[b : b + 1, i : i + chunk],
                        n_samples, n_classes,
                    )
                )
            outs.append(torch.cat(parts, dim=-1))
    return torch.cat(outs, dim=0)
