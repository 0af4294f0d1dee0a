"""Generate golden fixtures by running the reference renderer itself.

Runs nanodrr's `render(..., backend="torch")` (the reference's PyTorch
backend, src/nanodrr/drr/backends.py:9-63) on CPU, imported from a checkout
of the reference with the annotation/IO-only dependencies replaced by the
stand-ins in `_refstubs/` (jaxtyping, torchio, roma, platformdirs — none of
them touch the rendering arithmetic). Poses are passed as explicit 4x4
matrices built by `nanodrr_gb300.geometry.make_rt_inv`, so roma is never
needed. Writes `*.npz` next to this script: inputs and reference outputs.

Cases mirror the reference's own tests:
  impulse.npz   — tests/drr/test_renderer.py:8-91 (unit impulse, one ray,
                  1001 samples, integral = 1 ± 1e-3);
  random32.npz  — tests/drr/test_fused.py:11-47 subject/camera: forward
                  (persp/ortho × C=1/3), pose, volume and intrinsics
                  gradients (:68-144), pose-batch broadcast (:192-209), in
                  float32 and float64;
  phantom40.npz — a 40³ version of the seeded CT phantom, C=1 and C=8;
  homography.npz — the reference's 2-D intrinsics resample
                  (src/nanodrr/camera/homography.py:6-58) in float64: output
                  and gradients to the image and both inverse intrinsics;
  ncc.npz       — the reference's NormalizedCrossCorrelation2d
                  (src/nanodrr/metrics/ncc.py) in float64, global and 5x5
                  patches: scores and gradients to both images.

Usage: python tests/golden/make_golden.py /path/to/reference [case ...]
(or NANODRR_REFERENCE=/path/to/reference python tests/golden/make_golden.py)
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
if len(sys.argv) > 1:
    REF = Path(sys.argv[1])
elif os.environ.get("NANODRR_REFERENCE"):
    REF = Path(os.environ["NANODRR_REFERENCE"])
else:
    sys.exit("usage: make_golden.py /path/to/nanodrr-checkout [case ...] (or set NANODRR_REFERENCE)")

os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
sys.dont_write_bytecode = True
sys.path[:0] = [str(HERE / "_refstubs"), str(REF / "src"), str(REPO)]

import numpy as np  # noqa: E402
import torch  # noqa: E402

from nanodrr.data.subject import Subject as RefSubject  # noqa: E402
from nanodrr.drr.renderer import render as ref_render  # noqa: E402

from nanodrr_gb300.geometry import make_k_inv, make_rt_inv  # noqa: E402
from nanodrr_gb300.phantom import make_phantom  # noqa: E402


def ref_subject(image, label, voxel_to_world, n_classes):
    world_to_voxel = torch.linalg.inv(voxel_to_world)
    return RefSubject(
        imagedata=image,
        labeldata=label,
        voxel_to_world=voxel_to_world,
        world_to_voxel=world_to_voxel,
        voxel_to_grid=RefSubject._make_voxel_to_grid(image.shape).to(image.dtype),
        isocenter=torch.zeros(3, dtype=image.dtype),
        max_label=n_classes - 1,
        convert_to_mu=False,
    )


def impulse():
    image = torch.zeros(1, 1, 3, 3, 3)
    image[0, 0, 1, 1, 1] = 1.0
    v2w = torch.eye(4)
    v2w[:3, 3] = -1.0
    sub = ref_subject(image, torch.zeros_like(image), v2w, 1)
    k_inv = torch.eye(3)[None]
    rt_inv = torch.eye(4)[None]
    sdd = torch.tensor([1.0])
    src = torch.tensor([[[-1.5, 0.0, 0.0]]])
    tgt = torch.tensor([[[1.5, 0.0, 0.0]]])
    out = ref_render(sub, k_inv, rt_inv, sdd, 1, 1, n_samples=1001, src=src, tgt=tgt, backend="torch")
    np.savez_compressed(
        HERE / "impulse.npz",
        vol=image[0, 0].numpy(),
        voxel_to_world=v2w.numpy(),
        world_to_voxel=torch.linalg.inv(v2w).numpy(),
        k_inv=k_inv.numpy(),
        rt_inv=rt_inv.numpy(),
        sdd=sdd.numpy(),
        src=src.numpy(),
        tgt=tgt.numpy(),
        n_samples=np.int64(1001),
        out=out.detach().numpy(),
    )
    print("impulse", float(out))


def random32():
    size, C = 32, 3
    torch.manual_seed(0)
    image = torch.rand(1, 1, size, size, size, dtype=torch.float32)
    label = (torch.rand_like(image) * C).floor().clamp(max=C - 1)
    v2w = torch.eye(4)
    v2w[:3, 3] = -(size - 1) / 2
    H = W = 16
    sdd_f = 100.0
    k_inv = make_k_inv(sdd_f, 1.0, 1.0, 0.0, 0.0, H, W)
    rt1 = make_rt_inv(torch.tensor([[5.0, -3.0, 8.0]]), torch.tensor([[1.0, 80.0, -2.0]]), "AP", torch.zeros(3))
    rt2 = make_rt_inv(
        torch.tensor([[5.0, -3.0, 8.0], [25.0, 4.0, -6.0]]),
        torch.tensor([[1.0, 80.0, -2.0], [-3.0, 78.0, 5.0]]),
        "AP",
        torch.zeros(3),
    )
    sdd = torch.tensor([sdd_f])
    n = 200
    res = dict(
        vol=image[0, 0].numpy(),
        lab=label[0, 0].numpy().astype(np.uint8),
        voxel_to_world=v2w.numpy(),
        world_to_voxel=torch.linalg.inv(v2w).numpy(),
        k_inv=k_inv.numpy(),
        rt_inv=rt1.numpy(),
        rt_inv2=rt2.numpy(),
        sdd=sdd.numpy(),
        n_samples=np.int64(n),
        height=np.int64(H),
        width=np.int64(W),
    )
    torch.manual_seed(1)
    w_pose = torch.randn(1, 1, H, W)
    torch.manual_seed(2)
    w_vol1 = torch.randn(1, 1, H, W)
    torch.manual_seed(2)
    w_vol3 = torch.randn(1, C, H, W)
    torch.manual_seed(3)
    w_intr = torch.randn(1, 1, H, W)
    res.update(w_pose=w_pose.numpy(), w_vol1=w_vol1.numpy(), w_vol3=w_vol3.numpy(), w_intr=w_intr.numpy())

    for dt, tag in ((torch.float32, "f32"), (torch.float64, "f64")):
        for c in (1, C):
            lab = label if c > 1 else torch.zeros_like(image)
            sub = ref_subject(image.to(dt), lab.to(dt), v2w.to(dt), c)
            for ortho in (False, True):
                out = ref_render(
                    sub, k_inv.to(dt), rt1.to(dt), sdd.to(dt), H, W, n_samples=n, orthographic=ortho, backend="torch"
                )
                res[f"fwd_{'ortho' if ortho else 'persp'}_c{c}_{tag}"] = out.detach().numpy()
            out = ref_render(sub, k_inv.to(dt), rt2.to(dt), sdd.to(dt), H, W, n_samples=n, backend="torch")
            res[f"bcast_c{c}_{tag}"] = out.detach().numpy()
            # volume gradient (test_fused.py:103-122)
            sub._image_hu = sub._image_hu.detach().requires_grad_(True)
            out = ref_render(sub, k_inv.to(dt), rt1.to(dt), sdd.to(dt), H, W, n_samples=n, backend="torch")
            (out * (w_vol1 if c == 1 else w_vol3).to(dt)).sum().backward()
            res[f"gvol_c{c}_{tag}"] = sub._image_hu.grad[0, 0].numpy()
        sub = ref_subject(image.to(dt), torch.zeros_like(image).to(dt), v2w.to(dt), 1)
        for ortho in (False, True):
            rt = rt1.to(dt).clone().requires_grad_(True)
            out = ref_render(sub, k_inv.to(dt), rt, sdd.to(dt), H, W, n_samples=n, orthographic=ortho, backend="torch")
            (out * w_pose.to(dt)).sum().backward()
            res[f"grt_{'ortho' if ortho else 'persp'}_{tag}"] = rt.grad.numpy()
        k = k_inv.to(dt).clone().requires_grad_(True)
        s = sdd.to(dt).clone().requires_grad_(True)
        out = ref_render(sub, k, rt1.to(dt), s, H, W, n_samples=n, backend="torch")
        (out * w_intr.to(dt)).sum().backward()
        res[f"gk_{tag}"] = k.grad.numpy()
        res[f"gsdd_{tag}"] = s.grad.numpy()
    np.savez_compressed(HERE / "random32.npz", **res)
    print("random32", sorted(k for k in res if k.startswith(("fwd", "g", "bcast"))))


def phantom40():
    size = 40
    ph = make_phantom((size, size, size), (128.0 / size,) * 3, seed=0)
    vol, lab = ph.mu, ph.label
    sx = 128.0 / size
    v2w = torch.eye(4)
    v2w[0, 0] = v2w[1, 1] = v2w[2, 2] = sx
    v2w[:3, 3] = -(size - 1) / 2 * sx
    H = W = 24
    k_inv = make_k_inv(1020.0, 1.4 * 200 / W, 1.4 * 200 / H, 0.0, 0.0, H, W)
    rt = make_rt_inv(torch.zeros(1, 3), torch.tensor([[0.0, 600.0, 0.0]]), "AP", torch.zeros(3))
    rt_rot = make_rt_inv(torch.tensor([[20.0, -15.0, 10.0]]), torch.tensor([[10.0, 590.0, -20.0]]), "AP", torch.zeros(3))
    sdd = torch.tensor([1020.0])
    n = 300
    res = dict(
        vol=vol.numpy(),
        lab=lab.numpy(),
        voxel_to_world=v2w.numpy(),
        world_to_voxel=torch.linalg.inv(v2w).numpy(),
        k_inv=k_inv.numpy(),
        rt_inv=rt.numpy(),
        rt_inv_rot=rt_rot.numpy(),
        sdd=sdd.numpy(),
        n_samples=np.int64(n),
        height=np.int64(H),
        width=np.int64(W),
    )
    for dt, tag in ((torch.float32, "f32"), (torch.float64, "f64")):
        for c in (1, 8):
            labt = lab.to(dt) if c > 1 else torch.zeros_like(vol, dtype=dt)
            sub = ref_subject(vol.to(dt)[None, None], labt[None, None], v2w.to(dt), c)
            for name, r in (("id", rt), ("rot", rt_rot)):
                out = ref_render(sub, k_inv.to(dt), r.to(dt), sdd.to(dt), H, W, n_samples=n, backend="torch")
                res[f"fwd_{name}_c{c}_{tag}"] = out.detach().numpy()
    np.savez_compressed(HERE / "phantom40.npz", **res)
    print("phantom40 done")


def homography():
    from nanodrr.camera.homography import resample as ref_resample

    g = torch.Generator().manual_seed(11)
    B, C, H, W = 2, 3, 17, 23
    img = torch.rand(B, C, H, W, generator=g, dtype=torch.float64)
    k_old = torch.stack([make_k_inv(1020.0, 1.4, 1.5, 2.0, -3.0, H, W, dtype=torch.float64)[0],
                         make_k_inv(1000.0, 1.3, 1.3, -1.0, 1.0, H, W, dtype=torch.float64)[0]])
    k_new = torch.stack([make_k_inv(1060.0, 1.2, 1.4, -2.0, 2.5, H, W, dtype=torch.float64)[0],
                         make_k_inv(990.0, 1.35, 1.25, 0.5, -0.5, H, W, dtype=torch.float64)[0]])
    go = torch.randn(B, C, H, W, generator=g, dtype=torch.float64)
    img_r, ko_r, kn_r = (x.clone().requires_grad_(True) for x in (img, k_old, k_new))
    out = ref_resample(img_r, ko_r, kn_r)
    (out * go).sum().backward()
    np.savez_compressed(
        HERE / "homography.npz", img=img.numpy(), k_inv_old=k_old.numpy(), k_inv_new=k_new.numpy(),
        go=go.numpy(), out=out.detach().numpy(), g_img=img_r.grad.numpy(), g_k_inv_old=ko_r.grad.numpy(),
        g_k_inv_new=kn_r.grad.numpy(),
    )
    print("homography done")


def ncc():
    from nanodrr.metrics.ncc import NormalizedCrossCorrelation2d as RefNCC

    g = torch.Generator().manual_seed(12)
    B, C, H, W = 3, 2, 20, 24
    x1 = torch.rand(B, C, H, W, generator=g, dtype=torch.float64)
    x2 = 0.6 * x1 + 0.4 * torch.rand(B, C, H, W, generator=g, dtype=torch.float64)
    go = torch.randn(B, generator=g, dtype=torch.float64)
    res = {"x1": x1.numpy(), "x2": x2.numpy(), "go": go.numpy()}
    for tag, patch in (("global", None), ("patch5", 5)):
        a, b = x1.clone().requires_grad_(True), x2.clone().requires_grad_(True)
        s = RefNCC(patch_size=patch)(a, b)
        (s * go).sum().backward()
        res[f"score_{tag}"] = s.detach().numpy()
        res[f"g1_{tag}"] = a.grad.numpy()
        res[f"g2_{tag}"] = b.grad.numpy()
    np.savez_compressed(HERE / "ncc.npz", **res)
    print("ncc done")


if __name__ == "__main__":
    torch.set_num_threads(min(8, os.cpu_count() or 1))
    cases = {"impulse": impulse, "random32": random32, "phantom40": phantom40, "homography": homography,
             "ncc": ncc}
    for name in (sys.argv[2:] or list(cases)):
        cases[name]()
