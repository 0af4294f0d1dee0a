"""Registration step (fwd + NCC + bwd to the se(3) 6-vector of each pose)
through the CUDA kernels, checked against central finite differences of the
same loss computed by the float64 oracle (h = 1e-3 rad / mm), as the
registration workload asks, and the volume gradient of the step against the
oracle's analytic backward."""

import numpy as np
import pytest
import torch
from _gpu_helpers import rel_maxabs

import nanodrr_gb300 as nd
from nanodrr_gb300 import phantom
from nanodrr_gb300.geometry import convert
from nanodrr_gb300.registration import NormalizedCrossCorrelation2d, Registration
from nanodrr_gb300.renderer import _make_src, _make_tgt
from oracle import ncc_oracle, render_oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _smooth_subject(size=40, spacing=3.0, seed=0):
    """Smooth random attenuation inside an ellipsoid that falls off to zero
    (a smooth volume keeps trilinear face-crossings from dominating the
    finite differences)."""
    rng = np.random.default_rng(seed)
    v = rng.random((size, size, size))
    for _ in range(4):
        for ax in range(3):
            v = (np.roll(v, 1, ax) + v + np.roll(v, -1, ax)) / 3.0
    c = (np.arange(size) - (size - 1) / 2) / (size / 2)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    env = np.clip(1.0 - (x**2 / 0.8 + y**2 / 0.6 + z**2 / 0.8), 0.0, None) ** 2
    vol = torch.from_numpy((0.02 * v * env).astype(np.float32))
    return nd.Subject.from_volume(vol.to(DEV), (spacing,) * 3, convert_to_mu=False)


def test_registration_pose_gradient_matches_central_differences():
    torch.manual_seed(0)
    sub = _smooth_subject()
    B, det, n = 2, 24, 160
    k_inv, sdd = phantom.detector(pixel=3.0, height=det, width=det)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = phantom.random_poses(B, seed=3, rot_deg=15.0, trans_mm=10.0).to(DEV)
    ncc = NormalizedCrossCorrelation2d()
    reg = Registration(sub, rt, k_inv, sdd, det, det, batch=B).to(DEV)
    with torch.no_grad():
        reg._rot.copy_(torch.tensor([[0.02, -0.01, 0.015], [-0.02, 0.01, 0.0]], device=DEV))
        reg._xyz.copy_(torch.tensor([[1.0, -0.5, 0.8], [0.3, 1.2, -1.0]], device=DEV))
        target = nd.render(sub, k_inv, rt, sdd, det, det, n_samples=n)
    loss = -ncc(reg(n_samples=n), target).sum()
    loss.backward()
    g = torch.cat([reg._rot.grad, reg._xyz.grad], dim=1).double().cpu()  # [B, 6]

    # float64 oracle of the same loss
    vol64 = sub.image[0, 0].detach().double().cpu()
    w2v = sub.world_to_voxel.double().cpu()
    tgt = _make_tgt(k_inv.double().cpu(), sdd.double().cpu(), det, det, "cpu", torch.float64)
    src = _make_src(False, tgt, sdd.double().cpu())
    rt64, piv, piv_inv = (t.double().cpu() for t in (reg.rt_inv, reg.pivot, reg.pivot_inv))
    target64 = target.double().cpu()
    base = torch.cat([reg._rot, reg._xyz], dim=1).detach().double().cpu()

    def loss64(params):
        T = convert(params[:, :3], params[:, 3:], "so3_log")
        pose = rt64 @ piv @ T @ piv_inv
        img = render_oracle(vol64, None, w2v, pose, src, tgt, n).reshape(B, 1, det, det)
        return -ncc_oracle(img, target64).sum()

    h = 1e-3
    fd = torch.zeros(B, 6, dtype=torch.float64)
    with torch.no_grad():
        for b in range(B):
            for j in range(6):
                e = torch.zeros_like(base)
                e[b, j] = h
                fd[b, j] = (loss64(base + e) - loss64(base - e)) / (2 * h)
    assert rel_maxabs(g, fd) < 1e-2, (g, fd)
    # and every component keeps its sign and size
    assert torch.allclose(g, fd, rtol=5e-2, atol=2e-2 * float(fd.abs().max()))


def test_registration_volume_gradient_matches_oracle_backward():
    sub = _smooth_subject(size=32, spacing=3.5, seed=1)
    B, det, n = 2, 20, 120
    k_inv, sdd = phantom.detector(pixel=3.0, height=det, width=det)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = phantom.random_poses(B, seed=5, rot_deg=15.0, trans_mm=10.0).to(DEV)
    vol = sub._image_hu.detach().clone().requires_grad_(True)
    sub._image_hu = vol
    w = torch.randn(B, 1, det, det, device=DEV)
    (nd.render(sub, k_inv, rt, sdd, det, det, n_samples=n) * w).sum().backward()
    vol64 = vol.detach()[0, 0].double().cpu().requires_grad_(True)
    tgt = _make_tgt(k_inv.double().cpu(), sdd.double().cpu(), det, det, "cpu", torch.float64)
    src = _make_src(False, tgt, sdd.double().cpu())
    out = render_oracle(vol64, None, sub.world_to_voxel.double().cpu(), rt.double().cpu(), src, tgt, n)
    (out.reshape(B, 1, det, det) * w.double().cpu()).sum().backward()
    assert rel_maxabs(vol.grad[0, 0], vol64.grad) < 1e-3


def test_graphed_step_replays_the_eager_step():
    from nanodrr_gb300.registration import GraphedStep

    sub = _smooth_subject(size=36, spacing=3.0, seed=2)
    B, det, n = 3, 24, 150
    k_inv, sdd = phantom.detector(pixel=3.0, height=det, width=det)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = phantom.random_poses(B, seed=8, rot_deg=15.0, trans_mm=10.0).to(DEV)
    with torch.no_grad():
        target = nd.render(sub, k_inv, rt, sdd, det, det, n_samples=n)
    vol = sub._image_hu.detach().clone().requires_grad_(True)
    sub._image_hu = vol
    reg = Registration(sub, rt, k_inv, sdd, det, det, batch=B).to(DEV)
    ncc = NormalizedCrossCorrelation2d()
    loss_fn = lambda img, tgt: -ncc(img, tgt).mean()  # noqa: E731
    new_rot = torch.tensor([[0.01, -0.02, 0.005]] * B, device=DEV)
    new_xyz = torch.tensor([[0.5, 1.0, -0.5]] * B, device=DEV)

    def eager():
        for p in (reg._rot, reg._xyz, vol):
            p.grad = None
        loss = loss_fn(reg(n_samples=n), target)
        loss.backward()
        return loss.detach().clone(), reg._rot.grad.clone(), reg._xyz.grad.clone(), vol.grad.clone()

    step = GraphedStep(reg, loss_fn, target, n_samples=n)
    with torch.no_grad():
        reg._rot.copy_(new_rot)
        reg._xyz.copy_(new_xyz)
    loss_g = step.replay().clone()
    g_rot, g_xyz, g_vol = (g.clone() for g in step.grads)
    ref = eager()
    assert torch.equal(loss_g, ref[0])
    assert torch.equal(g_rot, ref[1]) and torch.equal(g_xyz, ref[2])  # deterministic pose gradient
    assert rel_maxabs(g_vol, ref[3]) < 1e-5  # atomics: order-dependent rounding
