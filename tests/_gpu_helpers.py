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


def load_reference_triton():
    """The unmodified reference (baseline/_ref, installed by
    baseline/install_reference.py) with its Triton backend, or (None, why).
    Triton's bundled ptxas predates sm_103a, so the CUDA toolkit's ptxas is
    named for it (TRITON_PTXAS_PATH) unless one is set."""
    import os
    import shutil
    import sys
    from pathlib import Path

    ref_dir = Path(__file__).resolve().parents[1] / "baseline" / "_ref"
    if not (ref_dir / "nanodrr").is_dir():
        return None, "baseline/_ref is not installed"
    if "TRITON_PTXAS_PATH" not in os.environ:
        for cand in (shutil.which("ptxas"), "/usr/local/cuda/bin/ptxas"):
            if cand and Path(cand).exists():
                os.environ["TRITON_PTXAS_PATH"] = cand
                break
    try:
        import triton  # noqa: F401
    except Exception as e:
        return None, f"triton is not importable: {e}"
    if str(ref_dir) not in sys.path:
        sys.path.insert(0, str(ref_dir))
    try:
        from nanodrr.data import Subject as RefSubject
        from nanodrr.drr.renderer import _triton_available
        from nanodrr.drr.renderer import render as ref_render
    except Exception as e:
        return None, f"the reference does not import: {e}"
    if not _triton_available():
        return None, "the reference's Triton backend does not import"
    return {"Subject": RefSubject, "render": ref_render}, None
