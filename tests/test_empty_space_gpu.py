"""GPU checks of empty-space skipping: the occupancy grid and extent labels
against the float64 oracle, skipped renders equal to the plain march (image,
pose and camera gradients; volume gradients use the full window), the
proposal network's training kernels against the CPU oracle, and what the
trained network gains over the plain march."""

import numpy as np
import pytest
import torch
from _gpu_helpers import rel_maxabs

import nanodrr_gb300 as nd
from nanodrr_gb300 import _ffi, phantom
from nanodrr_gb300.empty_space import EmptySpace, OccupancyGrid, ProposalNetwork, extents, train_proposal
from nanodrr_gb300.raymarch import raymarch_backward, raymarch_forward
from nanodrr_gb300.renderer import _affine_product, _make_src, _make_tgt
from oracle import empty_space_oracle as eso

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _case(size=48, B=4, det=32, n=300, seed=4):
    ph = phantom.make_phantom((size, size, size), (128 / size,) * 3, seed=0)
    sub = ph.subject(device=DEV, with_labels=True)
    k_inv, sdd = phantom.detector(pixel=1.4 * 200 / det, height=det, width=det)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = phantom.random_poses(B, seed=seed).to(DEV)
    tgt = _make_tgt(k_inv, sdd, det, det, DEV, torch.float32).expand(B, -1, -1).contiguous()
    src = _make_src(False, tgt, sdd.expand(B)).contiguous()
    step = ((tgt - src).norm(dim=-1) / (n - 1)).contiguous()
    M = _affine_product(sub.world_to_voxel[:3], rt).contiguous()
    vol = sub.image[0, 0].contiguous()
    lab = ph.label.to(DEV).contiguous()
    return ph, sub, vol, lab, M, src, tgt, step, n, det, k_inv, sdd, rt


def test_occupancy_grid_matches_oracle():
    ph, sub, vol, *_ = _case(size=40)
    g = OccupancyGrid.build(vol, cell=4, max_dist=6)
    ref = eso.occupancy_grid(ph.mu.numpy(), 4, 6)
    assert g.grid.shape == ref.shape
    assert torch.equal(g.grid.cpu(), torch.from_numpy(ref))
    assert 0.0 < g.occupied_fraction() < 1.0


def test_extent_labels_match_oracle():
    ph, sub, vol, lab, M, src, tgt, step, n, det, *_ = _case(B=2, det=16)
    ext = extents(vol, M, src, tgt, step, n, det)
    ref = eso.extent(ph.mu.numpy(), M.cpu().numpy(), src.cpu().numpy(), tgt.cpu().numpy(), n)
    # t values are s / (S - 1) on both sides: equal up to fp32 rounding
    assert np.abs(ext.cpu().numpy() - ref).max() < 2e-6
    assert (ref[..., 0] <= ref[..., 1]).any() and (ref[..., 0] > ref[..., 1]).any()


@pytest.mark.parametrize("C", [1, 8])
@pytest.mark.parametrize("tile", [None, (8, 4, 4)])
def test_occupancy_skip_equals_plain_march(C, tile):
    ph, sub, vol, lab, M, src, tgt, step, n, det, *_ = _case()
    skip = EmptySpace.occupancy(vol, cell=4)
    stats = torch.zeros(4, dtype=torch.int64, device=DEV)
    plain, _ = raymarch_forward(vol, lab, M, src, tgt, step, n, C, det, tile=tile)
    fast, _ = raymarch_forward(vol, lab, M, src, tgt, step, n, C, det, tile=tile, skip=skip, stats=stats)
    assert rel_maxabs(fast, plain) < 1e-6
    rays, fallbacks, marched, boxed = stats.tolist()
    assert rays > 0 and fallbacks == 0 and marched < boxed
    go = torch.randn_like(plain)
    pg = raymarch_backward(go, vol, lab, M, src, tgt, step, n, C, det, False, True, tile=tile)
    sg = raymarch_backward(go, vol, lab, M, src, tgt, step, n, C, det, False, True, tile=tile, skip=skip)
    for name, a, b in zip(("gM", "gsrc", "gtgt", "gstep"), sg[1:], pg[1:]):
        assert rel_maxabs(a, b) < 1e-5, name
    # with a volume gradient the full window is used: identical to plain
    pv = raymarch_backward(go, vol, lab, M, src, tgt, step, n, C, det, True, False, tile=tile)
    sv = raymarch_backward(go, vol, lab, M, src, tgt, step, n, C, det, True, False, tile=tile, skip=skip)
    assert rel_maxabs(sv[0], pv[0]) < 1e-5


def test_proposal_training_kernels_match_cpu_oracle():
    rng = np.random.default_rng(1)
    net = ProposalNetwork(DEV, seed=3)
    X = torch.from_numpy(rng.standard_normal((300, 64)).astype(np.float32)).to(DEV)
    X[:, 54:] = 0
    T = torch.from_numpy(rng.uniform(0, 1, (300, 2)).astype(np.float32)).to(DEV)
    V = torch.from_numpy((rng.random(300) > 0.1).astype(np.uint8)).to(DEV)
    grads, loss = net.gradients(X, T, V, alpha=7.0)
    P = net.params.double().cpu().numpy()
    ref_loss, ref_g = eso.proposal_loss_grad(P, X.cpu().numpy(), T.cpu().numpy(), V.cpu().numpy(), 7.0, 1 / 300)
    assert abs(float(loss) - ref_loss) / ref_loss < 1e-4
    assert rel_maxabs(grads, ref_g) < 1e-4
    out = net.forward(X)
    assert rel_maxabs(out, eso.proposal_forward(P, X.cpu().numpy())) < 1e-5


def test_proposal_dataset_features_match_oracle():
    ph, sub, vol, lab, M, src, tgt, step, n, det, *_ = _case(B=2, det=16)
    ext = extents(vol, M, src, tgt, step, n, det)
    X, T, V = ProposalNetwork.dataset(vol, M, src, tgt, n, det, ext)
    Mn = M.double().cpu().numpy()
    p0 = np.einsum("bij,bnj->bni", Mn[:, :, :3], src.expand_as(tgt).double().cpu().numpy()) + Mn[:, None, :, 3]
    d = np.einsum("bij,bnj->bni", Mn[:, :, :3], (tgt - src).double().cpu().numpy())
    f, t0, t1, hit = eso.proposal_features(p0.reshape(-1, 3), d.reshape(-1, 3), vol.shape)
    assert np.array_equal(V.cpu().numpy().astype(bool), hit)
    assert np.abs(X.cpu().numpy()[hit] - f[hit]).max() < 1e-4


def test_trained_proposal_is_exact_and_gains_over_plain():
    ph, sub, vol, lab, M, src, tgt, step, n, det, k_inv, sdd, rt = _case(B=16, det=32, seed=7)
    net, hist = train_proposal(vol, M, src, tgt, step, n, det, epochs=150, batch=4096, lr=3e-3)
    assert hist[-1] < hist[0]
    # evaluate on held-out poses
    *_, M2, src2, tgt2, step2, _, _, _, _, _ = _case(B=4, det=32, seed=99)
    skip = EmptySpace.proposal(vol, net, cell=4, margin=2.0)
    untrained = EmptySpace.proposal(vol, ProposalNetwork(DEV, seed=5), cell=4, margin=2.0)
    plain, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det)
    res = {}
    for name, sk in (("trained", skip), ("untrained", untrained)):
        stats = torch.zeros(4, dtype=torch.int64, device=DEV)
        out, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det, skip=sk, stats=stats)
        assert rel_maxabs(out, plain) < 1e-6, name  # exact either way: the grid check guards it
        res[name] = stats.tolist()
    rays, fb, marched, boxed = res["trained"]
    assert fb / rays < 0.5
    assert marched < boxed
    # the trained network marches fewer samples than the untrained one
    assert marched < res["untrained"][2]


def test_render_with_empty_space_through_autograd():
    ph, sub, vol, lab, M, src, tgt, step, n, det, k_inv, sdd, rt = _case(B=3)
    rt1 = rt.clone().requires_grad_(True)
    img = nd.render(sub, k_inv, rt1, sdd, det, det, n_samples=n)
    w = torch.randn_like(img)
    (img * w).sum().backward()
    sub.empty_space = EmptySpace.occupancy(vol, cell=4)
    rt2 = rt.clone().requires_grad_(True)
    img2 = nd.render(sub, k_inv, rt2, sdd, det, det, n_samples=n)
    (img2 * w).sum().backward()
    assert rel_maxabs(img2, img) < 1e-6
    assert rel_maxabs(rt2.grad, rt1.grad) < 1e-5


def _trained(seed=7):
    ph, sub, vol, lab, M, src, tgt, step, n, det, k_inv, sdd, rt = _case(B=16, det=32, seed=seed)
    net, _ = train_proposal(vol, M, src, tgt, step, n, det, epochs=150, batch=4096, lr=3e-3)
    return vol, net, n, det


def test_trained_proposal_adjoint_equals_plain():
    """Skipped samples have eight zero corners, so the pose and camera
    gradients equal the plain march's. A sample with a tiny value near the
    body surface still has a full-size position gradient, so this is a
    stricter check than the image."""
    vol, net, n, det = _trained()
    *_, M2, src2, tgt2, step2, _, _, _, _, _ = _case(B=4, det=32, seed=99)
    skip = EmptySpace.proposal(vol, net, cell=4, margin=2.0)
    go = torch.randn(4, 1, det * det, device=DEV)
    plain, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det)
    fast, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det, skip=skip)
    # same non-zero samples; a sample split groups them differently (fp32 sums)
    assert rel_maxabs(fast, plain) < 1e-6
    pg = raymarch_backward(go, vol, vol, M2, src2, tgt2, step2, n, 1, det, False, True)
    sg = raymarch_backward(go, vol, vol, M2, src2, tgt2, step2, n, 1, det, False, True, skip=skip)
    for name, a, b in zip(("gM", "gsrc", "gtgt", "gstep"), sg[1:], pg[1:]):
        assert rel_maxabs(a, b) < 1e-5, name


@pytest.mark.parametrize("mode", ["occupancy", "proposal"])
def test_skip_windows_equal_in_kernel_skipping(mode):
    """Windows from ndrr_skip_windows give the in-kernel occupancy skip's
    samples (bitwise image, same counters) and the plain march's image (up
    to the grouping of fp32 sums under a sample split); the volume adjoint
    ignores them."""
    from nanodrr_gb300.raymarch import skip_windows

    vol, net, n, det = _trained()
    *_, M2, src2, tgt2, step2, _, _, _, _, _ = _case(B=4, det=32, seed=98)
    if mode == "occupancy":
        ahead = EmptySpace.occupancy(vol, cell=4, fused=False)
    else:
        ahead = EmptySpace.proposal(vol, net, cell=4, margin=2.0)
    plain, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det)
    s2 = torch.zeros(4, dtype=torch.int64, device=DEV)
    win = skip_windows(vol, M2, src2, tgt2, step2, n, det, ahead, stats=s2)
    b, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det, windows=win)
    assert rel_maxabs(b, plain) < 1e-6
    assert win.dtype == torch.int32 and win.shape == (4, det * det, 2)
    assert bool((win[..., 0] <= win[..., 1]).all())
    rays, fallbacks, marched, boxed = s2.tolist()
    assert rays > 0 and marched < boxed
    if mode == "occupancy":
        s1 = torch.zeros(4, dtype=torch.int64, device=DEV)
        a, _ = raymarch_forward(vol, vol, M2, src2, tgt2, step2, n, 1, det, skip=EmptySpace.occupancy(vol, cell=4),
                                stats=s1)
        assert torch.equal(a, b)
        assert s1.tolist() == s2.tolist() and fallbacks == 0
    go = torch.randn_like(plain)
    full = raymarch_backward(go, vol, vol, M2, src2, tgt2, step2, n, 1, det, True, False)
    skip = raymarch_backward(go, vol, vol, M2, src2, tgt2, step2, n, 1, det, True, False, windows=win)
    assert rel_maxabs(skip[0], full[0]) < 1e-5


def test_render_with_learned_proposal_through_autograd():
    vol, net, n, det = _trained()
    ph, sub, vol, lab, M, src, tgt, step, n, det, k_inv, sdd, rt = _case(B=3, seed=97)
    rt1 = rt.clone().requires_grad_(True)
    img = nd.render(sub, k_inv, rt1, sdd, det, det, n_samples=n)
    w = torch.randn_like(img)
    (img * w).sum().backward()
    sub.empty_space = EmptySpace.proposal(vol, net, cell=4, margin=2.0)
    rt2 = rt.clone().requires_grad_(True)
    img2 = nd.render(sub, k_inv, rt2, sdd, det, det, n_samples=n)
    (img2 * w).sum().backward()
    assert rel_maxabs(img2, img) < 1e-6
    assert rel_maxabs(rt2.grad, rt1.grad) < 1e-5


def test_render_rebuilds_a_stale_grid():
    """A grid built before the volume changed would skip samples that are no
    longer empty: render rebuilds it (in place) first, so skipping stays
    exact after an in-place edit of the volume, and a grid built from a copy
    is replaced by one of the rendered volume."""
    ph, sub, vol, lab, M, src, tgt, step, n, det, k_inv, sdd, rt = _case(B=3)
    sub.empty_space = EmptySpace.occupancy(vol.clone(), cell=4)
    grid = sub.empty_space.grid
    with torch.no_grad():
        a = nd.render(sub, k_inv, rt, sdd, det, det, n_samples=n)
    assert grid.describes(sub.image.reshape(sub.image.shape[-3:]))
    buf = grid.grid
    with torch.no_grad():
        sub.image[..., :4, :, :] += 0.05  # content in the air beside the body
        b = nd.render(sub, k_inv, rt, sdd, det, det, n_samples=n)
    assert grid.grid is buf  # rebuilt in place
    sub.empty_space = None
    with torch.no_grad():
        ref = nd.render(sub, k_inv, rt, sdd, det, det, n_samples=n)
    assert not torch.equal(a, ref)
    assert rel_maxabs(b, ref) < 1e-6


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("fused", [True, False])
def test_split_adjoint_pose_pass_uses_the_skip(fused, dtype):
    """gvol_mode 5: the pose pass (the gathers) honours the occupancy skip —
    as an in-kernel window or as sample windows — whose skipped samples carry
    no pose terms, while the positions-only scatter pass marches every
    sample: gM as without the skip (bitwise with sample windows and one thread
    per ray), the volume
    gradient equal to the slab-ordered adjoint's to rounding."""
    from nanodrr_gb300.raymarch import quad_volume

    ph, sub, vol, lab, M, src, tgt, step, n, det, *_ = _case(B=5)
    vol = vol.to(dtype)
    q = quad_volume(vol)
    go = torch.randn(5, 1, det * det, device=DEV, generator=torch.Generator(device=DEV).manual_seed(3))
    args = (go, vol, vol, M, src, tgt, step, n, 1, det, True, False)
    slab = raymarch_backward(*args, quad=q, gvol_mode=3)
    split = raymarch_backward(*args, quad=q, gvol_mode=5)
    again = raymarch_backward(*args, quad=q, gvol_mode=5)
    assert rel_maxabs(split[0], slab[0]) < 1e-5
    assert rel_maxabs(split[1], slab[1]) < 1e-5
    assert torch.equal(split[1], again[1])
    skip = EmptySpace.occupancy(vol, cell=4, fused=fused)
    sk = raymarch_backward(*args, quad=q, gvol_mode=5, skip=skip)
    # this small launch splits each ray's samples over several threads, whose
    # chunks follow the window: the pose gradient regroups
    assert rel_maxabs(sk[1], split[1]) < 1e-5
    assert rel_maxabs(sk[0], slab[0]) < 1e-5
    if not fused:  # one thread per ray: sample windows drop only zero terms
        one = raymarch_backward(*args, quad=q, gvol_mode=5, tile=(16, 8, 1))
        one_sk = raymarch_backward(*args, quad=q, gvol_mode=5, tile=(16, 8, 1), skip=skip)
        assert torch.equal(one_sk[1], one[1])


def test_slab_adjoint_takes_sample_windows_as_gather_windows():
    """With a volume gradient the slab-ordered adjoint of one channel takes
    the skip's sample windows as gather windows: samples outside are still
    scattered (the volume gradient needs every sample) but their zero
    corners are not loaded. gM bitwise as without windows (the skipped
    samples' pose terms are exact zeros), the volume gradient equal to
    rounding; gvol_mode 0 (auto) takes them as well."""
    from nanodrr_gb300.raymarch import quad_volume, skip_windows

    ph, sub, vol, lab, M, src, tgt, step, n, det, *_ = _case(B=5)
    q = quad_volume(vol)
    go = torch.randn(5, 1, det * det, device=DEV, generator=torch.Generator(device=DEV).manual_seed(5))
    args = (go, vol, vol, M, src, tgt, step, n, 1, det, True, False)
    full = raymarch_backward(*args, quad=q, gvol_mode=3)
    win = skip_windows(vol, M, src, tgt, step, n, det, EmptySpace.occupancy(vol, cell=4, fused=False))
    assert (win[..., 1] - win[..., 0]).sum() < (M.shape[0] * det * det * n)  # something is skipped
    gated = raymarch_backward(*args, quad=q, gvol_mode=3, windows=win)
    assert torch.equal(gated[1], full[1])
    assert rel_maxabs(gated[0], full[0]) < 1e-5
    auto = raymarch_backward(*args, quad=q, windows=win)
    assert torch.equal(auto[1], full[1])
    assert rel_maxabs(auto[0], full[0]) < 1e-5
