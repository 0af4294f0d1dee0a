"""NCC loss through the CUDA kernels against the reference's own scores and
gradients (tests/golden/ncc.npz, produced by running nanodrr's
NormalizedCrossCorrelation2d in float64), global and with 5 x 5 patches."""

from pathlib import Path

import numpy as np
import pytest
import torch
from _gpu_helpers import rel_maxabs

from nanodrr_gb300.registration import NormalizedCrossCorrelation2d

pytestmark = pytest.mark.gpu
DEV = "cuda"
GOLD = Path(__file__).resolve().parent / "golden" / "ncc.npz"


@pytest.mark.parametrize("tag,patch", [("global", None), ("patch5", 5)])
def test_ncc_matches_reference_golden(tag, patch):
    g = np.load(GOLD)
    x1 = torch.from_numpy(g["x1"]).float().to(DEV).requires_grad_(True)
    x2 = torch.from_numpy(g["x2"]).float().to(DEV).requires_grad_(True)
    s = NormalizedCrossCorrelation2d(patch_size=patch)(x1, x2)
    assert rel_maxabs(s, g[f"score_{tag}"]) < 1e-5
    (s * torch.from_numpy(g["go"]).float().to(DEV)).sum().backward()
    assert rel_maxabs(x1.grad, g[f"g1_{tag}"]) < 1e-4
    assert rel_maxabs(x2.grad, g[f"g2_{tag}"]) < 1e-4


def test_ncc_of_an_image_with_itself_is_one_and_deterministic():
    torch.manual_seed(0)
    x = torch.rand(4, 1, 300, 280, device=DEV)  # more than one 4096-pixel chunk per plane
    s = NormalizedCrossCorrelation2d()(x, x)
    assert float((s - 1).abs().max()) < 1e-5
    y = (x + 0.1 * torch.rand_like(x)).requires_grad_(True)
    grads = []
    for _ in range(2):
        y.grad = None
        NormalizedCrossCorrelation2d()(y, x).sum().backward()
        grads.append(y.grad.clone())
    assert torch.equal(grads[0], grads[1])
    ref = NormalizedCrossCorrelation2d()(y.detach().double().cpu().cuda(), x.double())  # float64 inputs are cast
    assert float((ref - NormalizedCrossCorrelation2d()(y.detach(), x).double()).abs().max()) < 1e-5
