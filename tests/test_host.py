"""Host-side logic on CPU: the render call's argument handling, pose/camera
construction, the Subject container, label packing and the phantom recipe.
Mirrors the reference's CPU tests (tests/drr/test_fused.py:229-251,
tests/geometry/test_transform.py, tests/geometry/test_se3.py)."""

import math

import numpy as np
import pytest
import torch

import nanodrr_gb300 as nd
from nanodrr_gb300 import geometry, phantom
from nanodrr_gb300.renderer import _make_src, _make_tgt, compact_label


def _subject(C=1):
    torch.manual_seed(0)
    img = torch.rand(1, 1, 8, 8, 8)
    lab = (torch.rand_like(img) * C).floor()
    eye = torch.eye(4)
    return nd.Subject(img, lab, eye, eye, nd.Subject._make_voxel_to_grid(img.shape), torch.zeros(3), C - 1,
                      convert_to_mu=False)


def test_invalid_n_samples_raises():
    with pytest.raises(ValueError, match="n_samples"):
        nd.render(_subject(), torch.eye(3)[None], torch.eye(4)[None], torch.ones(1), 4, 4, n_samples=1)


def test_unknown_backend_raises():
    with pytest.raises(ValueError, match="backend"):
        nd.render(_subject(), torch.eye(3)[None], torch.eye(4)[None], torch.ones(1), 4, 4, backend="torch")


def test_cpu_inputs_raise_instead_of_falling_back():
    with pytest.raises(RuntimeError, match="CUDA"):
        nd.render(_subject(), torch.eye(3)[None], torch.eye(4)[None], torch.ones(1), 4, 4)


def test_transform_point_identity_translation_composition():
    pts = torch.randn(2, 5, 3)
    torch.testing.assert_close(nd.transform_point(torch.eye(4).expand(2, 4, 4), pts), pts)
    T = torch.eye(4)
    T[:3, 3] = torch.tensor([1.0, -2.0, 0.5])
    torch.testing.assert_close(nd.transform_point(T[None], pts[:1]), pts[:1] + T[:3, 3])
    A = geometry.make_se3(geometry.rotvec_to_rotmat(torch.tensor([[0.1, 0.2, -0.3]])), torch.tensor([[1.0, 2, 3]]))
    B = geometry.make_se3(geometry.rotvec_to_rotmat(torch.tensor([[-0.4, 0.0, 0.2]])), torch.tensor([[0.0, -1, 2]]))
    torch.testing.assert_close(
        nd.transform_point(A @ B, pts[:1]), nd.transform_point(A, nd.transform_point(B, pts[:1])), atol=1e-5, rtol=1e-5
    )


def test_euler_rotations_are_orthonormal_and_ordered():
    ang = torch.tensor([[0.3, -0.2, 0.7]], dtype=torch.float64)
    for conv in ("ZXY", "XYZ", "zyx"):
        R = geometry.euler_to_rotmat(conv, ang)
        torch.testing.assert_close(R @ R.transpose(-1, -2), torch.eye(3, dtype=torch.float64)[None])
        assert torch.det(R).item() == pytest.approx(1.0)
    # intrinsic ZXY = Rz Rx Ry; extrinsic "yxz" applies the same rotations in reverse
    Rz = geometry._axis_rotation("z", ang[:, 0])
    Rx = geometry._axis_rotation("x", ang[:, 1])
    Ry = geometry._axis_rotation("y", ang[:, 2])
    torch.testing.assert_close(geometry.euler_to_rotmat("ZXY", ang), Rz @ Rx @ Ry)
    torch.testing.assert_close(geometry.euler_to_rotmat("yxz", ang[:, [2, 1, 0]]), Rz @ Rx @ Ry)


def test_rotvec_matches_axis_angle_and_is_smooth_at_zero():
    v = torch.tensor([[0.0, 0.0, math.pi / 3]], dtype=torch.float64)
    torch.testing.assert_close(geometry.rotvec_to_rotmat(v), geometry._axis_rotation("z", v[:, 2]))
    z = torch.zeros(1, 3, dtype=torch.float64, requires_grad=True)
    R = geometry.rotvec_to_rotmat(z)
    R.sum().backward()
    assert torch.isfinite(z.grad).all()
    torch.testing.assert_close(R.detach(), torch.eye(3, dtype=torch.float64)[None])


def test_make_k_inv_and_rays():
    k = nd.make_k_inv(1020.0, 1.4, 1.4, 0.0, 0.0, 200, 200)
    K = torch.tensor([[1020 / 1.4, 0, 100.0], [0, 1020 / 1.4, 100.0], [0, 0, 1]])
    torch.testing.assert_close(k[0], torch.linalg.inv(K), rtol=1e-6, atol=1e-9)
    tgt = _make_tgt(k, torch.tensor([1020.0]), 200, 200, "cpu", torch.float32)
    assert tgt.shape == (1, 40000, 3)
    assert torch.allclose(tgt[..., 2], torch.tensor(1020.0))
    src = _make_src(False, tgt, torch.tensor([1020.0]))
    assert src.shape == (1, 1, 3) and not src.any()
    srco = _make_src(True, tgt, torch.tensor([1020.0]))
    assert torch.allclose(srco[..., 2], torch.tensor(0.0))


def test_make_rt_inv_ap_looks_through_isocenter():
    rt = nd.make_rt_inv(torch.zeros(1, 3), torch.tensor([[0.0, 600.0, 0.0]]), "AP", torch.zeros(3))
    centre = rt[0, :3, 3]
    axis = rt[0, :3, 2]  # camera +z in world
    torch.testing.assert_close(centre, torch.tensor([0.0, 600.0, 0.0]))
    torch.testing.assert_close(axis, torch.tensor([0.0, -1.0, 0.0]))
    with pytest.raises(ValueError, match="orientation"):
        geometry.orientation_matrix("LR")


def test_subject_mu_cache_and_grid_affine():
    hu = torch.tensor([-2000.0, -1000.0, 0.0, 500.0, 1000.0]).reshape(1, 1, 1, 1, 5)
    eye = torch.eye(4)
    s = nd.Subject(hu, torch.zeros_like(hu), eye, eye, nd.Subject._make_voxel_to_grid(hu.shape), torch.zeros(3))
    mu = s.image.flatten()
    expect = torch.tensor([0.0, 0.0, nd.subject.MU_WATER, 0.0192 + 0.5 * (0.0573 - 0.0192), 0.0573])
    torch.testing.assert_close(mu, expect)
    s.mu_water = 0.02
    assert s.image.flatten()[2].item() == pytest.approx(0.02)
    A = nd.Subject._make_voxel_to_grid((1, 1, 4, 6, 8))
    # voxel centre 0 -> -1 + 1/S; voxel S-1 -> 1 - 1/S (align_corners=False)
    torch.testing.assert_close(A @ torch.tensor([0.0, 0, 0, 1]), torch.tensor([-1 + 1 / 8, -1 + 1 / 6, -1 + 1 / 4, 1]))
    with pytest.raises(TypeError, match="Unknown mu"):
        nd.Subject(hu, hu, eye, eye, eye, torch.zeros(3), bogus=1)


def test_subject_mu_follows_settings_and_hu_tensor():
    """The μ volume is rebuilt after a setting changes, after an in-place
    edit of the HU values, after a new HU tensor is assigned and after a
    dtype move; set_mu's result sticks until one of those happens."""
    hu = torch.tensor([-500.0, 0.0, 250.0, 800.0]).reshape(1, 1, 1, 1, 4)
    eye = torch.eye(4)
    s = nd.Subject(hu.clone(), torch.zeros_like(hu), eye, eye, eye, torch.zeros(3))
    first = s.image
    assert s.image is first  # reused
    s.hu_bone = 2000.0
    assert s.image is not first
    torch.testing.assert_close(s.image, nd.hu_to_mu(hu, hu_bone=2000.0))
    before = s.image
    s._image_hu.mul_(0.5)  # in-place edit of the HU values
    torch.testing.assert_close(s.image, nd.hu_to_mu(hu * 0.5, hu_bone=2000.0))
    assert s.image is not before
    s._image_hu = hu.clone() + 100.0  # a new HU tensor
    torch.testing.assert_close(s.image, nd.hu_to_mu(hu + 100.0, hu_bone=2000.0))
    w = torch.tensor(0.03, requires_grad=True)
    s.set_mu(mu_water=w)  # differentiable setting, stored settings unchanged
    assert s.mu_water == nd.subject.MU_WATER
    s.image.sum().backward()
    assert w.grad is not None and w.grad.item() != 0.0
    s.mu_bone = 0.06  # a setting change drops set_mu's result
    torch.testing.assert_close(s.image, nd.hu_to_mu(hu + 100.0, mu_bone=0.06, hu_bone=2000.0))
    s64 = s.double()
    assert s64.image.dtype == torch.float64
    s.convert_to_mu = False
    assert s.image is s._image_hu
    assert set(s.state_dict()) == {"_image_hu", "label", "voxel_to_world", "world_to_voxel", "voxel_to_grid",
                                   "world_to_grid", "isocenter"}


def test_hu_to_mu_piecewise_map_in_float64():
    hu = torch.tensor([float("nan"), -3000.0, -1000.0, -250.0, 0.0, 1e-3, 600.0, 4000.0], dtype=torch.float64)
    mu = nd.hu_to_mu(hu, 0.02, 0.05, 1500.0)
    h = hu.clamp(min=-1000.0)
    expect = torch.where(h <= 0, 0.02 * (1 + h / 1000), 0.02 + h / 1500.0 * 0.03).clamp(min=0.0)
    torch.testing.assert_close(mu, expect, equal_nan=True)
    assert torch.isnan(mu[0])


def test_drr_rays_follow_the_intrinsics():
    """DRR's src/tgt match the render call's ray construction and are rebuilt
    when an intrinsic is reassigned or edited in place; state dict holds the
    intrinsics only."""
    drr = nd.DRR.from_carm_intrinsics(1020.0, 1.4, 1.4, 0.0, 0.0, 6, 5)
    tgt = _make_tgt(drr.k_inv, drr.sdd, 6, 5, torch.device("cpu"), torch.float32)
    torch.testing.assert_close(drr.tgt, tgt)
    torch.testing.assert_close(drr.src, torch.zeros(1, 1, 3))
    assert drr.tgt is drr.tgt  # kept while nothing changed
    drr.sdd.mul_(0.5)
    torch.testing.assert_close(drr.tgt, _make_tgt(drr.k_inv, drr.sdd, 6, 5, torch.device("cpu"), torch.float32))
    drr.height = 3
    assert drr.tgt.shape == (1, 15, 3)
    drr.orthographic = True
    torch.testing.assert_close(drr.src, _make_src(True, drr.tgt, drr.sdd))
    drr.k_inv = drr.k_inv * 2.0
    torch.testing.assert_close(drr.tgt, _make_tgt(drr.k_inv, drr.sdd, 3, 5, torch.device("cpu"), torch.float32))
    assert set(drr.state_dict()) == {"k_inv", "sdd"}
    k = drr.k_inv.clone().requires_grad_(True)
    drr.k_inv = k
    assert drr.tgt is not drr.tgt and drr.tgt.grad_fn is not None  # a fresh graph per read
    assert drr.double().tgt.dtype == torch.float64


def test_from_volume_centres_the_volume():
    s = nd.Subject.from_volume(torch.zeros(4, 6, 8), spacing=(0.5, 1.0, 2.0))
    c = s.voxel_to_world @ torch.tensor([3.5, 2.5, 1.5, 1.0])
    torch.testing.assert_close(c[:3], torch.zeros(3))
    torch.testing.assert_close(s.isocenter, torch.zeros(3))


def test_compact_label_preserves_routing():
    lab = torch.tensor([-1.5, -0.5, 0.0, 0.7, 1.0, 2.9, 3.0, 7.0, 300.0]).reshape(1, 1, 1, 1, 9)
    eye = torch.eye(4)
    s = nd.Subject(torch.zeros_like(lab), lab, eye, eye, eye, torch.zeros(3), max_label=3)
    packed = compact_label(s)
    # trunc toward zero, then classes outside [0, 4) become 255 (dropped)
    assert packed.flatten().tolist() == [255, 0, 0, 0, 1, 2, 3, 255, 255]
    assert compact_label(s) is packed  # cached
    s.label.add_(0)  # in-place change bumps the version: re-packed
    assert compact_label(s) is not packed


def test_phantom_recipe_is_seeded_and_labelled():
    a = phantom.make_phantom((24, 24, 24), (128 / 24,) * 3, seed=3)
    b = phantom.make_phantom((24, 24, 24), (128 / 24,) * 3, seed=3)
    assert torch.equal(a.mu, b.mu) and torch.equal(a.label, b.label)
    assert set(np.unique(a.label.numpy()).tolist()) <= set(range(8))
    assert (a.mu[a.label == 0] == 0).all()  # air is exactly zero attenuation
    assert a.hu.max() >= 400 and a.hu.min() == -1000
    poses = phantom.random_poses(4, seed=1)
    assert poses.shape == (4, 4, 4)
    R = poses[:, :3, :3]
    torch.testing.assert_close(R @ R.transpose(-1, -2), torch.eye(3).expand(4, 3, 3), atol=1e-5, rtol=0)


def test_registration_rescale_scales_intrinsics_and_resolution():
    from nanodrr_gb300.registration import Registration

    sub = nd.Subject.from_volume(torch.zeros(4, 4, 4), (1.0, 1.0, 1.0), convert_to_mu=False)
    k_inv = geometry.make_k_inv(1000.0, 1.0, 1.0, 0.0, 0.0, 100, 80)
    rt = torch.eye(4)[None]
    reg = Registration(sub, rt, k_inv.clone(), torch.tensor([1000.0]), 100, 80)
    reg.rescale_(0.5)
    assert (reg.height, reg.width) == (50, 40)
    assert torch.allclose(reg.k_inv[0, 0, 0], k_inv[0, 0, 0] / 0.5)
    assert torch.allclose(reg.k_inv[0, 1, 1], k_inv[0, 1, 1] / 0.5)
    assert torch.equal(reg.k_inv[0, :, 2], k_inv[0, :, 2])


def test_occupancy_grid_knows_its_volume():
    """describes(): the same memory (tensor, view or detached alias) at the
    same version counter; an in-place edit, another tensor, or a source that
    is gone all call for a rebuild."""
    import weakref

    from nanodrr_gb300.empty_space import OccupancyGrid

    vol = torch.rand(1, 1, 6, 5, 4)
    view = vol.reshape(6, 5, 4)
    g = OccupancyGrid(torch.zeros(4, 4, 4, dtype=torch.uint8), 4, (6, 5, 4),
                      source=(weakref.ref(vol), view._version, view.data_ptr(), (6, 5, 4)))
    assert g.describes(view)
    assert g.describes(vol.detach()[0, 0])
    assert not g.describes(view.clone())
    vol.add_(1.0)
    assert not g.describes(view)
    g.source = (weakref.ref(vol), view._version, view.data_ptr(), (6, 5, 4))
    assert g.describes(vol.detach().reshape(6, 5, 4))
    other = torch.rand(6, 5, 4)
    g.source = (weakref.ref(other), other._version, other.data_ptr(), (6, 5, 4))
    del other
    assert not g.describes(view)
