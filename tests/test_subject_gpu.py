"""GPU checks of the subject and detector modules: the HU -> μ kernel
against the float64 formula of the reference (src/nanodrr/data/preprocess.py:
44-50), and `DRR(...)(subject, rt_inv)` against `render` (the reference's
module is a thin wrapper around the same call, src/nanodrr/drr/drr.py:67-89),
also after its intrinsics change."""

import ctypes

import pytest
import torch

import nanodrr_gb300 as nd
from nanodrr_gb300 import _ffi, phantom
from nanodrr_gb300.subject import _hu_to_mu_torch

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 2e-7), (torch.bfloat16, 8e-3), (torch.float16, 1e-3)])
def test_hu_to_mu_kernel_matches_float64_formula(dtype, tol):
    g = torch.Generator().manual_seed(0)
    hu = (torch.rand(1_000_003, generator=g, dtype=torch.float64) * 5000.0 - 2500.0).to(dtype)
    hu[:4] = torch.tensor([-1000.0, 0.0, 1500.0, -3000.0], dtype=dtype)
    mu = nd.hu_to_mu(hu.to(DEV), 0.0192, 0.0573, 1000.0)
    assert mu.dtype == dtype and mu.device.type == "cuda"
    ref = _hu_to_mu_torch(hu.double(), 0.0192, 0.0573, 1000.0)
    err = ((mu.double().cpu() - ref).abs() / ref.abs().max()).max().item()
    assert err <= tol, err
    assert mu[0].item() == 0.0 and mu[3].item() == 0.0  # air and below-air clamp to 0


def test_hu_to_mu_kernel_is_the_subject_path_and_validates():
    hu = torch.full((2, 3, 4), 100.0, device=DEV)
    s = nd.Subject.from_volume(hu)
    mu = s.image
    torch.testing.assert_close(mu, _hu_to_mu_torch(s._image_hu, 0.0192, 0.0573, 1000.0))
    lib = _ffi.load()
    rc = lib.ndrr_hu_to_mu(ctypes.c_void_p(hu.data_ptr()), 7, 24, 0.0192, 0.0573, 1000.0,
                           ctypes.c_void_p(hu.data_ptr()), None)
    assert rc == _ffi.NDRR_ERR_DTYPE
    rc = lib.ndrr_hu_to_mu(ctypes.c_void_p(hu.data_ptr()), 0, 24, 0.0192, 0.0573, 0.0,
                           ctypes.c_void_p(hu.data_ptr()), None)
    assert rc == _ffi.NDRR_ERR_INVALID_ARGUMENT


def test_drr_module_equals_render_and_follows_intrinsics():
    ph = phantom.make_phantom((40, 40, 40), (128 / 40,) * 3, seed=1)
    sub = ph.subject(device=DEV)
    drr = nd.DRR.from_carm_intrinsics(1020.0, 1.4 * 200 / 48, 1.4 * 200 / 48, 0.0, 0.0, 48, 40, device=DEV)
    rt = phantom.random_poses(3, seed=2).to(DEV)
    out = drr(sub, rt, n_samples=300)
    ref = nd.render(sub, drr.k_inv, rt, drr.sdd, 48, 40, n_samples=300)
    assert torch.equal(out, ref)
    # explicit rays through the render call give the same image
    ref_rays = nd.render(sub, drr.k_inv, rt, drr.sdd, 48, 40, n_samples=300, src=drr.src, tgt=drr.tgt)
    assert torch.equal(out, ref_rays)
    drr.sdd.mul_(0.9)  # in-place change of an intrinsic
    out2 = drr(sub, rt, n_samples=300)
    ref2 = nd.render(sub, drr.k_inv, rt, drr.sdd.clone(), 48, 40, n_samples=300)
    assert torch.equal(out2, ref2) and not torch.equal(out2, out)
    drr.width = 32  # a new detector size
    assert drr(sub, rt, n_samples=300).shape == (3, 1, 48, 32)


@pytest.mark.parametrize("ortho", [False, True])
@pytest.mark.parametrize("n_k,n_s", [(1, 1), (3, 1), (1, 3), (3, 3)])
def test_camera_ray_kernel_is_bitwise_the_tensor_expression(ortho, n_k, n_s):
    from nanodrr_gb300.renderer import _camera_rays, _make_src, _make_tgt

    g = torch.Generator().manual_seed(n_k * 10 + n_s)
    k = torch.stack([torch.linalg.inv(torch.tensor([[1000.0 + 50 * i, 0.3, 61.7], [0.0, 990.0 - 7 * i, 45.2],
                                                   [0.0, 0.0, 1.0]])) for i in range(n_k)])
    k = (k + 1e-6 * torch.randn(k.shape, generator=g)).to(DEV)
    s = (1020.0 + 30.0 * torch.rand(n_s, generator=g)).to(DEV)
    for H, W in [(7, 5), (200, 200), (1, 33)]:
        src, tgt = _camera_rays(k, s, H, W, ortho, torch.device(DEV), torch.float32)
        tgt_ref = _make_tgt(k, s, H, W, torch.device(DEV), torch.float32)
        src_ref = _make_src(ortho, tgt_ref, s)
        assert tgt.shape == tgt_ref.shape and src.shape == src_ref.shape
        assert torch.equal(tgt, tgt_ref) and torch.equal(src, src_ref)


def test_camera_rays_keep_the_intrinsics_gradient():
    from nanodrr_gb300.renderer import _camera_rays, _make_tgt

    k = torch.linalg.inv(torch.tensor([[[900.0, 0.0, 50.0], [0.0, 900.0, 40.0], [0.0, 0.0, 1.0]]])).to(DEV)
    k.requires_grad_(True)
    s = torch.tensor([1020.0], device=DEV)
    src, tgt = _camera_rays(k, s, 6, 4, False, torch.device(DEV), torch.float32)
    assert tgt.requires_grad  # the tensor expressions, not the kernel
    tgt.sum().backward()
    assert k.grad is not None and torch.isfinite(k.grad).all()
    with torch.no_grad():
        _, t2 = _camera_rays(k, s, 6, 4, False, torch.device(DEV), torch.float32)
    assert torch.equal(t2, _make_tgt(k.detach(), s, 6, 4, torch.device(DEV), torch.float32))


def test_graph_captured_render_follows_intrinsics_edits():
    ph = phantom.make_phantom((40, 40, 40), (128 / 40,) * 3, seed=3)
    sub = ph.subject(device=DEV)
    drr = nd.DRR.from_carm_intrinsics(1020.0, 1.4 * 200 / 48, 1.4 * 200 / 48, 0.0, 0.0, 48, 48, device=DEV)
    k, s = drr.k_inv.clone(), drr.sdd.clone()
    rt = phantom.random_poses(1, seed=4).to(DEV)
    call = lambda: nd.render(sub, k, rt, s, 48, 48, n_samples=300)  # noqa: E731
    with torch.no_grad():
        ref = call().clone()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                call()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            out = call()
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
        s.mul_(0.95)  # the graph reads the camera tensors on every replay
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(out, call())
        assert not torch.equal(out, ref)


def test_affine_cache_follows_pose_edits():
    """A repeated render without a gradient reuses the camera -> voxel affine
    of the same pose tensor; an in-place pose edit or a new tensor rebuilds
    it, and a render with a gradient never reads the cache."""
    ph = phantom.make_phantom((40, 40, 40), (128 / 40,) * 3, seed=5)
    sub = ph.subject(device=DEV)
    drr = nd.DRR.from_carm_intrinsics(1020.0, 1.4 * 200 / 32, 1.4 * 200 / 32, 0.0, 0.0, 32, 32, device=DEV)
    k, s = drr.k_inv, drr.sdd
    rt = phantom.random_poses(2, seed=6).to(DEV)
    with torch.no_grad():
        a = nd.render(sub, k, rt, s, 32, 32, n_samples=200)
        assert torch.equal(nd.render(sub, k, rt, s, 32, 32, n_samples=200), a)
        rt[:, :3, 3] += 5.0  # in place: the cached affine is stale
        c = nd.render(sub, k, rt, s, 32, 32, n_samples=200)
        assert torch.equal(c, nd.render(sub, k, rt.clone(), s, 32, 32, n_samples=200))
        assert not torch.equal(c, a)
    rtg = rt.clone().requires_grad_(True)
    g = nd.render(sub, k, rtg, s, 32, 32, n_samples=200)
    assert torch.equal(g.detach(), c)
    g.sum().backward()
    assert rtg.grad is not None and torch.isfinite(rtg.grad).all()
