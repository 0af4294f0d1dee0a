"""FP64-oracle parity at the sizes the benchmark is quoted on.

The CUDA path renders the benchmark's seeded 512^3 phantom (0.8 x 0.8 x 1.0
mm, float32) at its poses, 256^2 detector at 1.2 mm, 800 samples per ray,
and a seeded subset of each pose's rays is checked against the float64
restatement of the reference's PyTorch backend (nanodrr
src/nanodrr/drr/backends.py:9-63, autograd through it being that backend's
analytic backward) on the same float32 inputs cast to float64:

  - image: <= 1e-5 relative max-abs per pose (max |cuda - fp64| over the
    pose's rays / max |fp64|);
  - pose gradient (rows of rt_inv that reach the voxel affine) and volume
    gradient of a positively weighted sum of the rays: <= 1e-3 relative
    max-abs;
  - the plain march, the occupancy skip and the learned proposal, the skips
    also through their pose-only adjoint (sample windows);
  - the registration step's se(3) 6-vector gradient (pose kernel, render,
    NCC kernels, backward) against float64 autograd of the same loss at the
    same (float32) pose;
  - the per-label render of the 512 x 512 x 400 volume with 8 classes, f32
    and bf16 (the reference's channel-sum rule, tests/drr/test_fused.py:
    56-65: channel sum within the tolerance, fewer than 0.1 % of rays with a
    channel beyond it; bf16 within 1e-2);
  - a 1024^2 detector at 1000 samples per ray with the learned proposal;
  - the volume stored as bf16 and f16 (within 1e-2) and orthographic rays
    (within 1e-5).

Rays are subsets (ray lists through render(src=, tgt=)); one check ties the
subset render to the full-image render of the same poses.
"""

import pytest
import torch
from _gpu_helpers import rel_maxabs

import nanodrr_gb300 as nd
from nanodrr_gb300 import phantom
from nanodrr_gb300.empty_space import EmptySpace, train_proposal
from nanodrr_gb300.geometry import convert
from nanodrr_gb300.registration import NormalizedCrossCorrelation2d, Registration
from nanodrr_gb300.renderer import _affine_product, _make_src, _make_tgt
from oracle import ncc_oracle, render_oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"
SHAPE, SPACING = (512, 512, 512), (0.8, 0.8, 1.0)
DET, PIXEL, S = 256, 1.2, 800
RAYS = 2048  # per pose


def _subset(n_pix: int, B: int, seed: int) -> torch.Tensor:
    g = torch.Generator().manual_seed(seed)
    return torch.stack([torch.randperm(n_pix, generator=g)[:RAYS] for _ in range(B)])


def _rays(k_inv, sdd, det, idx):
    """Camera-space rays of the pixels idx [B, R] (float32 on the GPU, and
    float64 on the CPU from the same float32 intrinsics)."""
    tgt = _make_tgt(k_inv.to(DEV), sdd.to(DEV), det, det, DEV, torch.float32)[0]
    tgt = tgt[idx.to(DEV)].contiguous()  # [B, R, 3]
    src = torch.zeros(idx.shape[0], 1, 3, device=DEV)
    tgt64 = _make_tgt(k_inv.double(), sdd.double(), det, det, "cpu", torch.float64)[0][idx]
    return src, tgt, torch.zeros(idx.shape[0], 1, 3, dtype=torch.float64), tgt64


def _oracle(vol64, lab64, w2v64, rt64, src64, tgt64, n, C=1, weight=None):
    """float64 oracle per pose; with `weight` also the gradients of
    sum(weight * out) to rt_inv and the volume."""
    outs = []
    g_rt = torch.zeros_like(rt64)
    g_vol = torch.zeros_like(vol64) if weight is not None else None
    for b in range(rt64.shape[0]):
        rt_b = rt64[b : b + 1].clone().requires_grad_(weight is not None)
        v = vol64.requires_grad_(weight is not None)
        out = render_oracle(v, lab64, w2v64, rt_b, src64[b : b + 1], tgt64[b : b + 1], n, C)
        if weight is not None:
            (out * weight[b : b + 1]).sum().backward()
            g_rt[b] = rt_b.grad[0]
            g_vol += v.grad
            v.grad = None
        outs.append(out.detach())
        vol64.requires_grad_(False)
    return torch.cat(outs), g_rt, g_vol


def _per_pose_rel(out, ref):
    out = out.detach().double().cpu().reshape(ref.shape[0], -1)
    ref = ref.reshape(ref.shape[0], -1)
    return float(((out - ref).abs().amax(1) / ref.abs().amax(1)).max())


@pytest.fixture(scope="module")
def headline():
    ph = phantom.make_phantom(SHAPE, SPACING, seed=0, device=DEV)
    sub = ph.subject(device=DEV)
    del ph
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=PIXEL, height=DET, width=DET)
    rt = phantom.random_poses(32, seed=1)[:4]  # the benchmark's first poses
    idx = _subset(DET * DET, rt.shape[0], seed=11)
    src, tgt, src64, tgt64 = _rays(k_inv, sdd, DET, idx)
    vol = sub._image_hu.detach()[0, 0]
    # a quickly trained proposal network: the skip is exact whatever its quality
    rt_train = phantom.random_poses(4, seed=500).to(DEV)
    tgt_t = _make_tgt(k_inv.to(DEV), sdd.to(DEV), DET, DET, DEV, torch.float32).expand(4, -1, -1).contiguous()
    src_t = torch.zeros(4, DET * DET, 3, device=DEV)
    step_t = ((tgt_t - src_t).norm(dim=-1) / (S - 1)).contiguous()
    Mt = _affine_product(sub.world_to_voxel[:3], rt_train).contiguous()
    net, _ = train_proposal(vol, Mt, src_t, tgt_t, step_t, S, DET, epochs=8, batch=65536)
    skips = {
        "plain": None,
        "occupancy": EmptySpace.occupancy(vol, cell=4),
        "learned": EmptySpace.proposal(vol, net, cell=4, margin=2.0),
    }
    vol64 = vol.double().cpu()
    w2v64 = sub.world_to_voxel.double().cpu()
    weight = 0.5 + torch.rand(rt.shape[0], 1, RAYS, generator=torch.Generator().manual_seed(3), dtype=torch.float64)
    ref, g_rt64, g_vol64 = _oracle(vol64, None, w2v64, rt.double(), src64, tgt64, S, weight=weight)
    return dict(sub=sub, k_inv=k_inv.to(DEV), sdd=sdd.to(DEV), rt=rt.to(DEV), idx=idx, src=src, tgt=tgt,
                skips=skips, ref=ref, g_rt64=g_rt64, g_vol64=g_vol64, weight=weight.float().to(DEV))


def _render_subset(h, rt, skip):
    h["sub"].empty_space = skip
    try:
        out = nd.render(h["sub"], h["k_inv"], rt, h["sdd"], RAYS // 64, 64, n_samples=S, src=h["src"], tgt=h["tgt"])
    finally:
        h["sub"].empty_space = None
    return out.reshape(rt.shape[0], 1, RAYS)


@pytest.mark.parametrize("method", ["plain", "occupancy", "learned"])
def test_headline_image_within_1e5_of_fp64(headline, method):
    h = headline
    with torch.no_grad():
        out = _render_subset(h, h["rt"], h["skips"][method])
    err = _per_pose_rel(out, h["ref"])
    assert err <= 1e-5, (method, err)


def test_headline_subset_render_is_the_full_image_render(headline):
    h = headline
    with torch.no_grad():
        full = nd.render(h["sub"], h["k_inv"], h["rt"], h["sdd"], DET, DET, n_samples=S).reshape(4, -1)
        sub = _render_subset(h, h["rt"], None)[:, 0]
    picked = torch.gather(full, 1, h["idx"].to(DEV))
    # the same per-sample arithmetic; the sums differ in order only (the
    # 8192-ray list is a small launch that splits each ray 16 ways)
    assert rel_maxabs(sub, picked) <= 5e-6


@pytest.mark.parametrize("method", ["plain", "learned"])
def test_headline_pose_and_volume_gradients_within_1e3_of_fp64(headline, method):
    h = headline
    sub = h["sub"]
    vol = sub._image_hu.detach().clone().requires_grad_(True)
    keep = sub._image_hu
    sub._image_hu = vol
    try:
        rt = h["rt"].clone().requires_grad_(True)
        (_render_subset(h, rt, h["skips"][method]) * h["weight"]).sum().backward()
    finally:
        sub._image_hu = keep
    assert rel_maxabs(rt.grad[:, :3], h["g_rt64"][:, :3]) <= 1e-3
    assert rel_maxabs(vol.grad[0, 0], h["g_vol64"]) <= 1e-3


@pytest.mark.parametrize("method", ["plain", "occupancy", "learned"])
def test_headline_pose_only_adjoint_within_1e3_of_fp64(headline, method):
    """Without a volume gradient the skips also shorten the adjoint (sample
    windows): its pose gradient is still the full march's."""
    h = headline
    rt = h["rt"].clone().requires_grad_(True)
    (_render_subset(h, rt, h["skips"][method]) * h["weight"]).sum().backward()
    assert rel_maxabs(rt.grad[:, :3], h["g_rt64"][:, :3]) <= 1e-3


def test_headline_registration_se3_gradient_within_1e3_of_fp64(headline):
    """The registration step at the benchmark volume and sample count (a 64^2
    detector over the same field of view, two poses): NCC against targets at
    held-out poses, gradient to each pose's rotation vector and translation
    against float64 autograd of the same composition and loss."""
    h = headline
    sub = h["sub"]
    det, B = 64, 2
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=PIXEL * DET / det, height=det, width=det)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = h["rt"][:B]
    held = rt @ convert(torch.tensor([[0.03, -0.02, 0.01], [-0.01, 0.02, 0.03]]),
                        torch.tensor([[2.0, -1.0, 3.0], [-2.0, 1.5, 1.0]]), "so3_log").to(DEV)
    with torch.no_grad():
        target = nd.render(sub, k_inv, held, sdd, det, det, n_samples=S)
    reg = Registration(sub, rt, k_inv, sdd, det, det, batch=B).to(DEV)
    with torch.no_grad():
        reg._rot.copy_(torch.tensor([[0.01, 0.02, -0.01], [0.02, -0.01, 0.0]]))
        reg._xyz.copy_(torch.tensor([[1.0, 0.5, -1.0], [-0.5, 1.0, 0.5]]))
    ncc = NormalizedCrossCorrelation2d()
    (-ncc(reg(n_samples=S), target).sum()).backward()
    g = torch.cat([reg._rot.grad, reg._xyz.grad], dim=1).double().cpu()

    params = torch.cat([reg._rot, reg._xyz], dim=1).detach().double().cpu().requires_grad_(True)
    rt64, piv, piv_inv = (t.detach().double().cpu() for t in (reg.rt_inv, reg.pivot, reg.pivot_inv))
    exact = rt64 @ piv @ convert(params[:, :3], params[:, 3:], "so3_log") @ piv_inv
    # identical inputs: the float32 pose the renderer received (the pose
    # kernel's output), differentiated through the exact composition — the
    # loss's gradient moves by ~1e-3 when only the pose is rounded to float32
    pose = exact + (reg.pose.detach().double().cpu() - exact).detach()
    tgt64 = _make_tgt(k_inv.double().cpu(), sdd.double().cpu(), det, det, "cpu", torch.float64)
    src64 = _make_src(False, tgt64, sdd.double().cpu())
    vol64 = sub._image_hu.detach()[0, 0].double().cpu()
    img = render_oracle(vol64, None, sub.world_to_voxel.double().cpu(), pose, src64, tgt64, S)
    loss = -ncc_oracle(img.reshape(B, 1, det, det), target.double().cpu()).sum()
    loss.backward()
    assert rel_maxabs(g, params.grad) <= 1e-3, (g, params.grad)


@pytest.fixture(scope="module")
def labelled():
    ph = phantom.make_phantom((400, 512, 512), SPACING, seed=0, device=DEV)
    subs = {dt: ph.subject(dtype=dt, with_labels=True, device=DEV) for dt in (torch.float32, torch.bfloat16)}
    lab64 = ph.label.double().cpu()
    vol64 = ph.mu.double().cpu()
    del ph
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=PIXEL, height=DET, width=DET)
    rt = phantom.random_poses(32, seed=1)[:2]
    idx = _subset(DET * DET, 2, seed=12)
    src, tgt, src64, tgt64 = _rays(k_inv, sdd, DET, idx)
    w2v64 = subs[torch.float32].world_to_voxel.double().cpu()
    ref, _, _ = _oracle(vol64, lab64, w2v64, rt.double(), src64, tgt64, S, C=8)
    return dict(subs=subs, k_inv=k_inv.to(DEV), sdd=sdd.to(DEV), rt=rt.to(DEV), src=src, tgt=tgt, ref=ref)


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.bfloat16, 1e-2)])
def test_per_label_render_at_config_size(labelled, dtype, tol):
    L = labelled
    with torch.no_grad():
        out = nd.render(L["subs"][dtype], L["k_inv"], L["rt"], L["sdd"], RAYS // 64, 64, n_samples=S,
                        src=L["src"], tgt=L["tgt"]).reshape(2, 8, RAYS)
    ref = L["ref"]
    out = out.double().cpu()
    total_err = _per_pose_rel(out.sum(1), ref.sum(1))
    assert total_err <= tol, total_err
    scale = ref.abs().amax(dim=(1, 2), keepdim=True)
    bad = ((out - ref).abs() / scale > tol).any(dim=1)  # rays with any channel beyond the tolerance
    assert bad.double().mean().item() < 1e-3, bad.double().mean().item()


def test_learned_proposal_1024_detector_within_tolerances(headline):
    """1024^2 detector at 1000 samples per ray with the learned proposal: the
    image within 1e-5, the pose (pose-only adjoint with windows) and volume
    gradients within 1e-3 of the float64 oracle."""
    h = headline
    sub = h["sub"]
    det, n, B = 1024, 1000, 2
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=PIXEL * DET / det, height=det, width=det)
    rt = phantom.random_poses(8, seed=7)[:B]
    idx = _subset(det * det, B, seed=13)
    src, tgt, src64, tgt64 = _rays(k_inv, sdd, det, idx)
    weight = 0.5 + torch.rand(B, 1, RAYS, generator=torch.Generator().manual_seed(4), dtype=torch.float64)
    vol64 = sub._image_hu.detach()[0, 0].double().cpu()
    ref, g_rt64, g_vol64 = _oracle(vol64, None, sub.world_to_voxel.double().cpu(), rt.double(), src64, tgt64, n,
                                   weight=weight)
    k_inv, sdd, rt, w = k_inv.to(DEV), sdd.to(DEV), rt.to(DEV), weight.float().to(DEV)
    sub.empty_space = h["skips"]["learned"]
    vol = sub._image_hu.detach().clone().requires_grad_(True)
    keep = sub._image_hu
    try:
        rt_p = rt.clone().requires_grad_(True)
        out = nd.render(sub, k_inv, rt_p, sdd, RAYS // 64, 64, n_samples=n, src=src, tgt=tgt).reshape(B, 1, RAYS)
        assert _per_pose_rel(out, ref) <= 1e-5
        (out * w).sum().backward()
        assert rel_maxabs(rt_p.grad[:, :3], g_rt64[:, :3]) <= 1e-3
        sub._image_hu = vol
        rt_v = rt.clone().requires_grad_(True)
        out = nd.render(sub, k_inv, rt_v, sdd, RAYS // 64, 64, n_samples=n, src=src, tgt=tgt).reshape(B, 1, RAYS)
        (out * w).sum().backward()
        assert rel_maxabs(rt_v.grad[:, :3], g_rt64[:, :3]) <= 1e-3
        assert rel_maxabs(vol.grad[0, 0], g_vol64) <= 1e-3
    finally:
        sub.empty_space = None
        sub._image_hu = keep


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
def test_headline_16bit_volume_within_1e2_of_fp64(headline, dtype):
    """The benchmark volume stored as bf16 / f16 (its quad layout of 16-bit
    values, fp32 accumulation): the image within 1e-2 of the float64 oracle
    of the float32 volume."""
    h = headline
    s16 = nd.Subject.from_volume(h["sub"]._image_hu.detach()[0, 0].to(dtype), SPACING, convert_to_mu=False)
    with torch.no_grad():
        out = nd.render(s16, h["k_inv"], h["rt"], h["sdd"], RAYS // 64, 64, n_samples=S, src=h["src"], tgt=h["tgt"])
    assert out.dtype == dtype
    err = _per_pose_rel(out.reshape(4, 1, RAYS).float(), h["ref"])
    assert err <= 1e-2, err


def test_headline_orthographic_image_within_1e5_of_fp64(headline):
    """Parallel rays of the same pixel subset (src = tgt - (0, 0, sdd), one
    source per ray) at the benchmark size: the image within 1e-5 of the
    float64 oracle."""
    h = headline
    sub = h["sub"]
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=PIXEL, height=DET, width=DET)
    tgt = h["tgt"]
    src = tgt.clone()
    src[..., 2] -= h["sdd"][0]
    tgt64 = _make_tgt(k_inv.double(), sdd.double(), DET, DET, "cpu", torch.float64)[0][h["idx"]]
    src64 = tgt64.clone()
    src64[..., 2] -= float(sdd[0])
    vol64 = sub._image_hu.detach()[0, 0].double().cpu()
    ref, _, _ = _oracle(vol64, None, sub.world_to_voxel.double().cpu(), h["rt"].double().cpu(), src64, tgt64, S)
    with torch.no_grad():
        out = nd.render(sub, h["k_inv"], h["rt"], h["sdd"], RAYS // 64, 64, n_samples=S, src=src, tgt=tgt)
    assert float(ref.abs().max()) > 0
    err = _per_pose_rel(out.reshape(4, 1, RAYS), ref)
    assert err <= 1e-5, err
