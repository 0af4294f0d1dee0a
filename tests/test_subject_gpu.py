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
