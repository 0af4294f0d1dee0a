"""Parity with the reference's own fused Triton kernel, run unmodified from
baseline/_ref through its render(..., backend="triton") (nanodrr
src/nanodrr/drr/renderer.py:84-98, src/nanodrr/drr/_fused.py:415-567) on the
same inputs: images within 1e-4 (the reference's own rule for its fused
kernel, tests/drr/test_fused.py:56-65: channel sums, and fewer than 0.1 % of
pixels off in any channel), pose and volume gradients within 1e-3
(test_fused.py:82-144). Skipped, with the reason, where the reference or
Triton cannot run."""

import pytest
import torch
from _gpu_helpers import assert_render_parity, load_reference_triton, rays_for, rel_maxabs, subject_from_arrays

import nanodrr_gb300 as nd
from nanodrr_gb300 import phantom

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def ref():
    r, why = load_reference_triton()
    if r is None:
        pytest.skip(why)
    return r


def _ref_subject(ref, sub):
    """The reference's Subject over the same tensors as `sub`."""
    return ref["Subject"](
        imagedata=sub._image_hu,
        labeldata=sub.label,
        voxel_to_world=sub.voxel_to_world,
        world_to_voxel=sub.world_to_voxel,
        voxel_to_grid=sub.voxel_to_grid,
        isocenter=sub.isocenter,
        max_label=sub.n_classes - 1,
        convert_to_mu=False,
    )


@pytest.mark.parametrize("orthographic", [False, True])
@pytest.mark.parametrize("n_classes", [1, 3])
def test_forward_matches_reference_triton(ref, random32, orthographic, n_classes):
    g = random32
    sub = subject_from_arrays(g["vol"], g["lab"], g["voxel_to_world"], n_classes)
    rsub = _ref_subject(ref, sub)
    k_inv, rt, sdd, H, W = rays_for(g)
    n = int(g["n_samples"])
    with torch.no_grad():
        mine = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=n, orthographic=orthographic)
        theirs = ref["render"](rsub, k_inv, rt, sdd, H, W, n_samples=n, orthographic=orthographic, backend="triton")
    assert_render_parity(theirs, mine, n_classes, tol=1e-4)


def test_gradients_match_reference_triton_on_a_phantom(ref):
    """128^3 phantom (the CPU-runnable configuration's volume), four random
    poses, 200^2 detector at 1.4 mm, 500 samples: image, pose gradient and
    volume gradient of a weighted image sum."""
    ph = phantom.make_phantom((128, 128, 128), (1.0, 1.0, 1.0), seed=0, device=DEV)
    sub = ph.subject(device=DEV)
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=1.4, height=200, width=200)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = phantom.random_poses(4, seed=3).to(DEV)
    w = torch.rand(4, 1, 200, 200, device=DEV, generator=torch.Generator(DEV).manual_seed(0))
    results = []
    for which in ("mine", "theirs"):
        vol = sub._image_hu.detach().clone().requires_grad_(True)
        sub._image_hu = vol
        r = rt.clone().requires_grad_(True)
        if which == "mine":
            img = nd.render(sub, k_inv, r, sdd, 200, 200, n_samples=500)
        else:
            img = ref["render"](_ref_subject(ref, sub), k_inv, r, sdd, 200, 200, n_samples=500, backend="triton")
        (img * w).sum().backward()
        results.append((img.detach(), r.grad[:, :3].clone(), vol.grad.clone()))
    (im, gr, gv), (it, grt, gvt) = results
    assert_render_parity(it, im, 1, tol=1e-4)
    assert rel_maxabs(gr, grt) < 1e-3
    assert rel_maxabs(gv, gvt) < 1e-3
