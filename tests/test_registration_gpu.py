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
    # a volume update between replays (as an optimiser makes) reaches the
    # graph: its quad copy is rebuilt in place, also after an eager render
    # replaced the subject's cached copy
    with torch.no_grad():
        vol.mul_(1.5)
        vol[:, :, 10:20] += 0.01
    ref2 = eager()
    with torch.no_grad():
        vol.mul_(0.9)
    ref3 = eager()
    loss_3 = step.replay().clone()
    assert torch.equal(loss_3, ref3[0])
    assert torch.equal(step.grads[0], ref3[1]) and torch.equal(step.grads[1], ref3[2])
    assert not torch.equal(ref2[0], ref3[0])
    # a different volume tensor cannot be followed by the graph: replay refuses
    sub._image_hu = vol.detach().clone().requires_grad_(True)
    with pytest.raises(RuntimeError, match="captured"):
        step.replay()


def _torch_pose64(rot, xyz, rt, piv, piv_inv):
    from nanodrr_gb300.geometry import mm_small

    T = convert(rot, xyz, "so3_log")
    return mm_small(mm_small(mm_small(rt, piv), T), piv_inv)


@pytest.mark.parametrize("rows", [1, 5])
@pytest.mark.parametrize("scale", [1e-8, 1e-3, 0.05, 1.2])
def test_so3_pose_kernel_matches_torch_float64(rows, scale):
    """ndrr_pose_so3_fwd/bwd against the torch composition of the reference's
    Registration.pose in float64 (rotation vectors from the identity's
    Taylor range to 1.2 rad; a broadcast single-row parameter and one row per
    pose)."""
    from nanodrr_gb300.registration import so3_pose

    g = torch.Generator().manual_seed(int(scale * 1e9) % 1000 + rows)
    B = 5
    rt = phantom.random_poses(B, seed=11).double()
    c = torch.randn(B, 3, generator=g, dtype=torch.float64) * 20
    piv = Registration._make_translation(c)
    piv_inv = Registration._make_translation(-c)
    rot = (torch.randn(rows, 3, generator=g, dtype=torch.float64) * scale)
    xyz = torch.randn(rows, 3, generator=g, dtype=torch.float64) * 5
    gp = torch.randn(B, 4, 4, generator=g, dtype=torch.float64)
    # float32-representable inputs: both sides see the same numbers
    rt, piv, piv_inv, rot, xyz, gp = (t.float().double() for t in (rt, piv, piv_inv, rot, xyz, gp))

    r64, x64 = rot.clone().requires_grad_(True), xyz.clone().requires_grad_(True)
    ref = _torch_pose64(r64, x64, rt, piv, piv_inv)
    (ref * gp).sum().backward()

    rf, xf = rot.float().to(DEV).requires_grad_(True), xyz.float().to(DEV).requires_grad_(True)
    out = so3_pose(rf, xf, rt.float().to(DEV), piv.float().to(DEV), piv_inv.float().to(DEV))
    (out * gp.float().to(DEV)).sum().backward()
    assert out.shape == (B, 4, 4)
    assert rel_maxabs(out, ref.detach()) < 1e-6
    # the kernel evaluates in float64: the gradients agree to the float32
    # rounding of its outputs
    assert rel_maxabs(rf.grad, r64.grad) < 1e-5
    assert rel_maxabs(xf.grad, x64.grad) < 1e-5


def test_so3_pose_rejects_bad_shapes():
    from nanodrr_gb300.registration import so3_pose

    rt = phantom.random_poses(3, seed=1).to(DEV)
    piv = torch.eye(4, device=DEV).expand(3, 4, 4).contiguous()
    with pytest.raises(ValueError):
        so3_pose(torch.zeros(2, 3, device=DEV), torch.zeros(2, 3, device=DEV), rt, piv, piv)
    with pytest.raises(ValueError):
        so3_pose(torch.zeros(3, 3, device=DEV), torch.zeros(3, 3, device=DEV), rt, piv[:2], piv)


def test_registration_pose_uses_the_kernel_and_matches_host_composition():
    sub = _smooth_subject(size=16)
    B = 3
    rt = phantom.random_poses(B, seed=4).to(DEV)
    k_inv, sdd = phantom.detector(pixel=3.0, height=8, width=8)
    reg = Registration(sub, rt, k_inv.to(DEV), sdd.to(DEV), 8, 8, batch=B).to(DEV)
    with torch.no_grad():
        reg._rot.copy_(torch.tensor([[0.1, -0.2, 0.05], [0.0, 0.0, 0.0], [1e-5, 2e-5, -1e-5]], device=DEV))
        reg._xyz.copy_(torch.tensor([[1.0, 2.0, -3.0], [0.5, 0.0, 0.0], [0.0, -1.0, 0.0]], device=DEV))
    P = reg.pose
    assert P.requires_grad
    ref = _torch_pose64(reg._rot.detach().double().cpu(), reg._xyz.detach().double().cpu(),
                        reg.rt_inv.double().cpu(), reg.pivot.double().cpu(), reg.pivot_inv.double().cpu())
    assert rel_maxabs(P.detach(), ref) < 1e-6


def test_rescale_renders_at_the_new_resolution():
    sub = _smooth_subject(size=24)
    rt = phantom.random_poses(2, seed=5).to(DEV)
    k_inv, sdd = phantom.detector(pixel=3.0, height=16, width=16)
    reg = Registration(sub, rt, k_inv.to(DEV), sdd.to(DEV), 16, 16, batch=2).to(DEV)
    with torch.no_grad():
        a = reg(n_samples=120)
        reg.rescale_(0.5)
        b = reg(n_samples=120)
        k2, _ = phantom.detector(pixel=6.0, height=8, width=8)
        ref = nd.render(sub, k2.to(DEV), reg.pose, reg.sdd, 8, 8, n_samples=120)
    assert a.shape[-2:] == (16, 16) and b.shape[-2:] == (8, 8)
    assert rel_maxabs(b, ref) < 1e-5
