"""Intrinsics resample (the reference's camera/homography.py `resample`)
through the CUDA kernels, against the golden output and gradients the
reference itself produced (tests/golden/homography.npz, float64)."""

from pathlib import Path

import numpy as np
import pytest
import torch
from _gpu_helpers import rel_maxabs

import nanodrr_gb300 as nd

pytestmark = pytest.mark.gpu
DEV = "cuda"
GOLD = Path(__file__).resolve().parent / "golden" / "homography.npz"


def test_resample_matches_reference_golden():
    g = np.load(GOLD)
    img = torch.from_numpy(g["img"]).float().to(DEV).requires_grad_(True)
    ko = torch.from_numpy(g["k_inv_old"]).float().to(DEV).requires_grad_(True)
    kn = torch.from_numpy(g["k_inv_new"]).float().to(DEV).requires_grad_(True)
    out = nd.resample(img, ko, kn)
    assert rel_maxabs(out, g["out"]) < 1e-5
    (out * torch.from_numpy(g["go"]).float().to(DEV)).sum().backward()
    assert rel_maxabs(img.grad, g["g_img"]) < 1e-5
    # intrinsics gradients pass through the perspective divide and the 3x3
    # inverse in float32: relative to their scale
    assert rel_maxabs(ko.grad, g["g_k_inv_old"]) < 1e-3
    assert rel_maxabs(kn.grad, g["g_k_inv_new"]) < 1e-3


def test_resample_identity_and_shift():
    torch.manual_seed(0)
    img = torch.rand(2, 3, 20, 30, device=DEV)
    k = nd.make_k_inv(1000.0, 1.0, 1.0, 0.0, 0.0, 20, 30, device=DEV).expand(2, 3, 3)
    assert rel_maxabs(nd.resample(img, k, k), img) < 1e-6
    # moving the principal point by one pixel shifts the image by one column
    k2 = nd.make_k_inv(1000.0, 1.0, 1.0, 1.0, 0.0, 20, 30, device=DEV).expand(2, 3, 3)
    out = nd.resample(img, k, k2)
    assert rel_maxabs(out[..., 1:], img[..., :-1]) < 1e-5
    assert float(out[..., 0].abs().max()) < 1e-5


def test_resample_homography_gradient_is_deterministic_and_rejects_bad_input():
    torch.manual_seed(1)
    img = torch.rand(3, 2, 17, 19, device=DEV)
    ko = nd.make_k_inv(1000.0, 1.2, 1.1, 0.5, -0.5, 17, 19, device=DEV).expand(3, 3, 3).clone().requires_grad_(True)
    kn = nd.make_k_inv(980.0, 1.1, 1.2, -0.5, 0.5, 17, 19, device=DEV).expand(3, 3, 3)
    grads = []
    for _ in range(2):
        ko.grad = None
        nd.resample(img, ko, kn).square().sum().backward()
        grads.append(ko.grad.clone())
    assert torch.equal(grads[0], grads[1])
    with pytest.raises(ValueError, match="float32"):
        nd.resample(img.double(), ko.detach().double(), kn.double())
