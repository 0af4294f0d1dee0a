"""Shared helpers for the GPU tests: build subjects from golden arrays and
compare results the way the reference's parity tests do."""

from __future__ import annotations

import numpy as np
import torch

import nanodrr_gb300 as nd


def subject_from_arrays(vol, lab, voxel_to_world, C, dtype=torch.float32, device="cuda"):
    img = torch.as_tensor(vol).to(device=device, dtype=dtype)[None, None]
    if C > 1:
        labt = torch.as_tensor(lab).to(device=device, dtype=torch.float32)[None, None]
    else:
        labt = torch.zeros(img.shape, device=device, dtype=torch.float32)
    v2w64 = torch.as_tensor(voxel_to_world).double()
    return nd.Subject(
        img,
        labt,
        v2w64.float().to(device),
        torch.linalg.inv(v2w64).float().to(device),
        nd.Subject._make_voxel_to_grid(img.shape).to(device),
        torch.zeros(3, device=device),
        max_label=C - 1,
        convert_to_mu=False,
    )


def rel_maxabs(out, ref) -> float:
    out = torch.as_tensor(out).detach().double().cpu()
    ref = torch.as_tensor(ref).detach().double().cpu()
    return float((out - ref).abs().max() / ref.abs().max().clamp_min(1e-30))


def assert_render_parity(ref, out, n_classes, tol=1e-5):
    """Reference parity rule (tests/drr/test_fused.py:56-65): C == 1 compares
    max-abs / scale; C > 1 compares the channel sum and allows < 0.1 % of
    pixels to differ (label routing is discontinuous at label boundaries)."""
    ref = torch.as_tensor(ref).double().cpu()
    out = torch.as_tensor(out).double().cpu()
    scale = ref.abs().max()
    if n_classes == 1:
        err = ((ref - out).abs().max() / scale).item()
        assert err < tol, err
    else:
        err = ((ref.sum(1) - out.sum(1)).abs().max() / scale).item()
        assert err < tol, err
        bad = ((ref - out).abs().amax(dim=1) / scale) > tol
        assert bad.float().mean().item() < 1e-3, bad.float().mean().item()


def rays_for(g, rt_key="rt_inv", ortho=False, device="cuda", dtype=torch.float32):
    H, W = int(g["height"]), int(g["width"])
    k_inv = torch.as_tensor(g["k_inv"]).to(device, dtype)
    sdd = torch.as_tensor(g["sdd"]).to(device, dtype)
    rt = torch.as_tensor(g[rt_key]).to(device, dtype)
    return k_inv, rt, sdd, H, W


def np64(t) -> np.ndarray:
    return torch.as_tensor(t).detach().double().cpu().numpy()
