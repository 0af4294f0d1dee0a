"""GPU parity of the CUDA ray march against the reference's outputs (golden
fixtures generated by the reference) and the float64 oracle.

Mirrors the reference's parity suite (tests/drr/test_fused.py:68-226) and
known-answer test (tests/drr/test_renderer.py:52-91), with these
tolerances: float32 forward within 1e-5 relative max-abs of the float64
reference, gradients within 1e-3, bf16/f16 volumes within 1e-2.
"""

import ctypes

import numpy as np
import pytest
import torch
from _gpu_helpers import assert_render_parity, np64, rays_for, rel_maxabs, subject_from_arrays

import nanodrr_gb300 as nd
from nanodrr_gb300 import _ffi
from nanodrr_gb300.raymarch import raymarch_backward, raymarch_forward
from oracle import march_numpy, march_numpy_adjoint

pytestmark = pytest.mark.gpu
DEV = "cuda"


def test_single_ray_integral_equals_one(impulse):
    g = impulse
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    out = nd.render(
        sub,
        torch.as_tensor(g["k_inv"]).to(DEV),
        torch.as_tensor(g["rt_inv"]).to(DEV),
        torch.as_tensor(g["sdd"]).to(DEV),
        1,
        1,
        n_samples=1001,
        src=torch.as_tensor(g["src"]).to(DEV),
        tgt=torch.as_tensor(g["tgt"]).to(DEV),
    )
    assert float(out) == pytest.approx(1.0, rel=1e-3, abs=1e-3)
    assert float(out) == pytest.approx(float(g["out"].squeeze()), rel=1e-5)


@pytest.mark.parametrize("orthographic", [False, True])
@pytest.mark.parametrize("n_classes", [1, 3])
def test_forward_matches_reference(random32, orthographic, n_classes):
    g = random32
    sub = subject_from_arrays(g["vol"], g["lab"], g["voxel_to_world"], n_classes)
    k_inv, rt, sdd, H, W = rays_for(g)
    out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=int(g["n_samples"]), orthographic=orthographic)
    assert out.shape == (1, n_classes, H, W)
    key = f"fwd_{'ortho' if orthographic else 'persp'}_c{n_classes}"
    assert_render_parity(g[key + "_f64"], out, n_classes, tol=1e-5)
    assert_render_parity(g[key + "_f32"], out, n_classes, tol=1e-4)


@pytest.mark.parametrize("orthographic", [False, True])
def test_pose_gradients_match_reference(random32, orthographic):
    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    k_inv, rt, sdd, H, W = rays_for(g)
    rt = rt.clone().requires_grad_(True)
    out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=int(g["n_samples"]), orthographic=orthographic)
    (out * torch.as_tensor(g["w_pose"]).to(DEV)).sum().backward()
    ref = g[f"grt_{'ortho' if orthographic else 'persp'}_f64"][0, :3]
    assert rel_maxabs(rt.grad[0, :3], ref) < 1e-3


@pytest.mark.parametrize("n_classes", [1, 3])
def test_volume_gradients_match_reference(random32, n_classes):
    g = random32
    sub = subject_from_arrays(g["vol"], g["lab"], g["voxel_to_world"], n_classes)
    sub._image_hu = sub._image_hu.detach().requires_grad_(True)
    k_inv, rt, sdd, H, W = rays_for(g)
    out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=int(g["n_samples"]))
    w = g["w_vol1"] if n_classes == 1 else g["w_vol3"]
    (out * torch.as_tensor(w).to(DEV)).sum().backward()
    assert rel_maxabs(sub._image_hu.grad[0, 0], g[f"gvol_c{n_classes}_f64"]) < 1e-3


def test_intrinsics_gradients_match_reference(random32):
    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    k_inv, rt, sdd, H, W = rays_for(g)
    k = k_inv.clone().requires_grad_(True)
    s = sdd.clone().requires_grad_(True)
    out = nd.render(sub, k, rt, s, H, W, n_samples=int(g["n_samples"]))
    (out * torch.as_tensor(g["w_intr"]).to(DEV)).sum().backward()
    assert rel_maxabs(k.grad, g["gk_f64"]) < 1e-3
    assert rel_maxabs(s.grad, g["gsdd_f64"]) < 1e-3


def test_pose_gradients_bitwise_deterministic(random32):
    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    k_inv, rt_inv, sdd, H, W = rays_for(g)
    w = torch.as_tensor(g["w_pose"]).to(DEV)
    grads = []
    for _ in range(3):
        rt = rt_inv.clone().requires_grad_(True)
        (nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200) * w).sum().backward()
        grads.append(rt.grad.clone())
    torch.testing.assert_close(grads[0], grads[1], rtol=0, atol=0)
    torch.testing.assert_close(grads[0], grads[2], rtol=0, atol=0)


@pytest.mark.parametrize("n_classes", [1, 3])
def test_pose_batch_broadcast(random32, n_classes):
    g = random32
    sub = subject_from_arrays(g["vol"], g["lab"], g["voxel_to_world"], n_classes)
    k_inv, rt2, sdd, H, W = rays_for(g, rt_key="rt_inv2")
    out = nd.render(sub, k_inv, rt2, sdd, H, W, n_samples=200)
    assert out.shape == (2, n_classes, H, W)
    assert_render_parity(g[f"bcast_c{n_classes}_f64"], out, n_classes, tol=1e-5)


def test_out_of_range_labels_are_safe(random32):
    g = random32
    lab = (np.arange(g["lab"].size).reshape(g["lab"].shape) % 5).astype(np.float32)
    sub = subject_from_arrays(g["vol"], lab, g["voxel_to_world"], 5)
    sub.n_classes = 3  # fewer channels than the label map holds
    k_inv, rt, sdd, H, W = rays_for(g)
    rt = rt.clone().requires_grad_(True)
    out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200)
    out.sum().backward()
    assert out.shape[1] == 3
    assert torch.isfinite(out).all() and torch.isfinite(rt.grad).all()
    # dropped labels contribute nothing: channel sum < unrouted integral
    total = nd.render(subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1), k_inv, rt.detach(), sdd, H, W,
                      n_samples=200)
    assert (out.sum(1) <= total[:, 0] * (1 + 1e-5) + 1e-6).all()


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
def test_half_volume_variants_within_1e_2(random32, dtype):
    g = random32
    for C in (1, 3):
        sub = subject_from_arrays(g["vol"], g["lab"], g["voxel_to_world"], C, dtype=dtype)
        k_inv, rt, sdd, H, W = rays_for(g)
        out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200)
        assert out.dtype == dtype
        assert_render_parity(g[f"fwd_persp_c{C}_f64"], out.float(), C, tol=1e-2)


@pytest.mark.parametrize("C", [1, 8])
@pytest.mark.parametrize("pose", ["id", "rot"])
def test_phantom_matches_reference(phantom40, C, pose):
    g = phantom40
    sub = subject_from_arrays(g["vol"], g["lab"], g["voxel_to_world"], C)
    k_inv, rt, sdd, H, W = rays_for(g, rt_key="rt_inv" if pose == "id" else "rt_inv_rot")
    out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=int(g["n_samples"]))
    assert_render_parity(g[f"fwd_{pose}_c{C}_f64"], out, C, tol=1e-5)


def test_deterministic_mode_rejects_volume_gradients(random32):
    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    sub._image_hu = sub._image_hu.detach().requires_grad_(True)
    k_inv, rt, sdd, H, W = rays_for(g)
    torch.use_deterministic_algorithms(True)
    try:
        out = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=50)
        with pytest.raises(RuntimeError, match="nondeterministic"):
            out.sum().backward()
        # pose-only gradients stay available (and bitwise deterministic)
        sub._image_hu = sub._image_hu.detach()
        rt = rt.clone().requires_grad_(True)
        nd.render(sub, k_inv, rt, sdd, H, W, n_samples=50).sum().backward()
        assert torch.isfinite(rt.grad).all()
    finally:
        torch.use_deterministic_algorithms(False)


def test_compiles_with_gradients(random32):
    """The custom ops trace opaquely under torch.compile (fake kernels)."""
    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    k_inv, rt_inv, sdd, H, W = rays_for(g)
    w = torch.as_tensor(g["w_pose"]).to(DEV)

    def f(rt):
        return nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200)

    rt = rt_inv.clone().requires_grad_(True)
    (f(rt) * w).sum().backward()
    torch._dynamo.reset()
    rt_c = rt_inv.clone().requires_grad_(True)
    (torch.compile(f, fullgraph=True, backend="aot_eager")(rt_c) * w).sum().backward()
    assert rel_maxabs(rt_c.grad[0, :3], rt.grad[0, :3]) < 1e-6


# ----------------------------------------------------------------- op level
def _smooth_noise(rng, shape, passes=3):
    """Random field smoothed by repeated 3-tap box filters: its trilinear
    interpolant has small gradient jumps across cell faces, so fp32-vs-fp64
    floor differences at faces barely move the pose gradient."""
    v = rng.random(shape)
    for _ in range(passes):
        for ax in range(3):
            v = (np.roll(v, 1, ax) + v + np.roll(v, -1, ax)) / 3.0
    return v.astype(np.float32)


def _random_case(seed, B=3, Hd=20, Wd=24, vol_shape=(40, 36, 44), ortho=False, C=1):
    rng = np.random.default_rng(seed)
    vol = _smooth_noise(rng, vol_shape)
    D, H, W = vol_shape
    # blocky labels (8-voxel blocks) with one out-of-range class value C
    z, y, x = np.meshgrid(np.arange(D) // 8, np.arange(H) // 8, np.arange(W) // 8, indexing="ij")
    lab = ((x + 2 * y + 3 * z + seed) % (C + 1)).astype(np.uint8)
    M = np.zeros((B, 3, 4), np.float32)
    for b in range(B):
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        M[b, :, :3] = q * rng.uniform(0.8, 1.2)
        M[b, :, 3] = np.array([W, H, D]) / 2 + rng.uniform(-3, 3, 3)
    N = Hd * Wd
    u, v = np.meshgrid(np.arange(Wd) - Wd / 2 + 0.5, np.arange(Hd) - Hd / 2 + 0.5)
    tgt = np.stack([u.ravel() * 2.0, v.ravel() * 2.0, np.full(N, 60.0)], -1)[None].repeat(B, 0).astype(np.float32)
    if ortho:
        src = tgt.copy()
        src[..., 2] = -60.0
    else:
        src = np.zeros((B, 1, 3), np.float32)
        src[..., 2] = -60.0
    step = (np.linalg.norm(tgt - src, axis=-1) / 199).astype(np.float32)
    return vol, lab, M, src, tgt, step, Wd


@pytest.mark.parametrize("ortho", [False, True])
@pytest.mark.parametrize("C", [1, 4])
def test_op_forward_and_adjoint_vs_numpy_oracle(ortho, C):
    n = 200
    vol, lab, M, src, tgt, step, width = _random_case(7, ortho=ortho, C=C)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    out, total = raymarch_forward(t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, C, width, with_total=True)
    ref = march_numpy(vol, lab, M, src, tgt, step, n, C)
    assert_render_parity(ref, out, C, tol=1e-5)
    ref1 = march_numpy(vol, lab, M, src, tgt, step, n, 1)
    assert rel_maxabs(total, ref1[:, 0]) < 1e-5
    rng = np.random.default_rng(3)
    go = rng.standard_normal(out.shape).astype(np.float32)
    gvol, gM, gsrc, gtgt, gstep = raymarch_backward(
        t(go), t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, C, width, True, True
    )
    rg = march_numpy_adjoint(go, vol, lab, M, src, tgt, step, n, C)
    # aggregated gradients: 1e-3 relative max-abs
    for name, mine, theirs in zip(("gvol", "gM"), (gvol, gM), rg[:2]):
        assert rel_maxabs(mine, theirs) < 1e-3, name
    per_ray = [("gtgt", gtgt, rg[3]), ("gstep", gstep, rg[4])]
    if ortho:
        per_ray.append(("gsrc", gsrc, rg[2]))  # one source per ray
    else:
        assert rel_maxabs(gsrc, rg[2]) < 1e-3  # one shared source per pose: aggregated
    # per-ray gradients: the trilinear gradient jumps across cell faces, so a
    # sample whose fp32 and fp64 positions straddle a face takes the other
    # one-sided value; at most 0.5 % of rays may differ by more than 1e-3
    # (relative to the largest), none by more than 5e-2
    for name, mine, theirs in per_ray:
        a = np64(mine).reshape(mine.shape[0], mine.shape[1], -1)
        b = np.asarray(theirs).reshape(a.shape)
        err = np.abs(a - b).max(-1) / np.abs(b).max()
        assert (err > 1e-3).mean() < 5e-3, name
        assert err.max() < 5e-2, name


@pytest.mark.parametrize("tile", [(8, 4, 1), (8, 8, 2), (16, 8, 4), (16, 16, 2), (32, 8, 1)])
def test_launch_shapes_agree_through_the_c_abi(tile):
    """Every tile shape / sample split gives the same image (C-ABI direct)."""
    n = 150
    vol, lab, M, src, tgt, step, width = _random_case(11, B=2, Hd=17, Wd=23, C=3)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    ref, _ = raymarch_forward(t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, 3, width)
    dv, dl, dM, ds, dt_, dst = t(vol), t(lab), t(M), t(src), t(tgt), t(step)
    out = torch.empty_like(ref)
    a = _ffi.RaymarchArgs()
    a.vol, a.vol_dtype, (a.D, a.H, a.W) = dv.data_ptr(), _ffi.NDRR_F32, vol.shape
    a.lab, a.lab_dtype, a.n_classes = dl.data_ptr(), _ffi.NDRR_U8, 3
    a.M, a.src, a.tgt, a.step = dM.data_ptr(), ds.data_ptr(), dt_.data_ptr(), dst.data_ptr()
    a.src_per_ray, a.B, a.N, a.width, a.n_samples = 0, 2, tgt.shape[1], width, n
    a.out, a.out_dtype = out.data_ptr(), _ffi.NDRR_F32
    a.tile_w, a.tile_h, a.sample_split = tile
    lib = _ffi.load()
    rc = lib.ndrr_raymarch_fwd(ctypes.byref(a), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, lib.ndrr_last_error()
    torch.cuda.synchronize()
    assert rel_maxabs(out, ref) < 1e-6


def test_linear_ray_list_and_per_ray_sources():
    """width that does not divide N -> flat ray list; per-ray sources."""
    n = 120
    vol, lab, M, src, tgt, step, width = _random_case(5, B=2, ortho=True)
    tgt, src, step = tgt[:, :451], src[:, :451], step[:, :451]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)  # noqa: E731
    out, _ = raymarch_forward(t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, 1, 0)
    ref = march_numpy(vol, lab, M, src, tgt, step, n, 1)
    assert rel_maxabs(out, ref) < 1e-5


def test_sample_window_restricts_the_march():
    n = 100
    vol, lab, M, src, tgt, step, width = _random_case(9, B=1)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)  # noqa: E731
    N = tgt.shape[1]
    win = np.zeros((1, N, 2), np.float32)
    win[..., 0] = 0.25
    win[..., 1] = 0.75
    out, _ = raymarch_forward(t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, 1, width, t_window=t(win))
    # only samples s with 0.25 <= s/(n-1) <= 0.75 count
    s = np.arange(n) / (n - 1)
    keep = (s >= 0.25) & (s <= 0.75)
    full = np.zeros((1, 1, N))
    for i in range(N):
        ts = s[keep]
        q = src[0, 0] + ts[:, None] * (tgt[0, i] - src[0, 0])
        p = q @ M[0, :, :3].T + M[0, :, 3]
        from oracle.numpy_oracle import _taps, _value

        vals, fx, fy, fz = _taps(vol.astype(np.float64), p[:, 0], p[:, 1], p[:, 2])
        full[0, 0, i] = _value(vals, fx, fy, fz).sum() * step[0, i]
    assert rel_maxabs(out, full) < 1e-5


def test_volume_adjoint_dot_product_identity():
    """<go, A vol> == <A^T go, vol>: the volume adjoint is the exact transpose."""
    n = 160
    vol, lab, M, src, tgt, step, width = _random_case(13, B=2, C=1)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    out, _ = raymarch_forward(t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, 1, width)
    go = torch.randn_like(out)
    gvol, *_ = raymarch_backward(go, t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, 1, width, True, False)
    lhs = (go.double() * out.double()).sum().item()
    rhs = (gvol.double() * t(vol).double()).sum().item()
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_empty_batch_and_no_rays():
    vol = torch.rand(4, 4, 4, device=DEV)
    M = torch.zeros(0, 3, 4, device=DEV)
    z3 = torch.zeros(0, 5, 3, device=DEV)
    out, _ = raymarch_forward(vol, vol, M, torch.zeros(0, 1, 3, device=DEV), z3, torch.zeros(0, 5, device=DEV), 10, 1, 5)
    assert out.shape == (0, 1, 5)


@pytest.mark.parametrize("C", [1, 4])
@pytest.mark.parametrize("cap,tile", [(0, (16, 8, 1)), (0, (8, 4, 1)), (0, (16, 16, 1)), (600, (16, 8, 1)),
                                      (60, (8, 8, 1))])
def test_brick_volume_gradient_matches_direct_and_oracle(C, cap, tile):
    """Per-slab shared-memory brick scatter == direct atomics == float64 oracle,
    including capacities small enough to force the fallback and L adaptation."""
    n = 180
    vol, lab, M, src, tgt, step, width = _random_case(21, B=2, Hd=19, Wd=26, C=C)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    out, _ = raymarch_forward(t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, C, width)
    go = torch.randn_like(out)
    args = (go, t(vol), t(lab), t(M), t(src), t(tgt), t(step), n, C, width, True, True)
    direct = raymarch_backward(*args, gvol_mode=_ffi.NDRR_GVOL_DIRECT, tile=tile)
    brick = raymarch_backward(*args, gvol_mode=_ffi.NDRR_GVOL_BRICK, brick_cap=cap, tile=tile)
    for name, x, y in zip(("gvol", "gM", "gsrc", "gtgt", "gstep"), brick, direct):
        assert rel_maxabs(x, y) < 1e-5, name
    ref = march_numpy_adjoint(np64(go), vol, lab, M, src, tgt, step, n, C)
    assert rel_maxabs(brick[0], ref[0]) < 1e-4
    assert rel_maxabs(brick[1], ref[1]) < 1e-3


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16, torch.float16])
@pytest.mark.parametrize("C", [1, 4])
def test_quad_layout_equals_plain_layout(dtype, C):
    """The quad layout holds exact copies of the corners: forward and pose
    gradient are bitwise equal to the plain layout's; the volume gradient
    (different atomic order, folded from quad entries) agrees to rounding."""
    from nanodrr_gb300.raymarch import quad_volume

    n = 170
    vol, lab, M, src, tgt, step, width = _random_case(31, B=2, Hd=21, Wd=27, C=C)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol).to(dtype)
    q = quad_volume(v)
    D, H, W = vol.shape
    assert q.numel() == (D + 4) * (H + 3) * (W + 3) * (16 if dtype == torch.float32 else 8)
    plain, _ = raymarch_forward(v, t(lab), t(M), t(src), t(tgt), t(step), n, C, width)
    quad, _ = raymarch_forward(v, t(lab), t(M), t(src), t(tgt), t(step), n, C, width, quad=q)
    assert torch.equal(plain, quad)
    go = torch.randn(plain.shape, device=DEV)
    gp = raymarch_backward(go, v, t(lab), t(M), t(src), t(tgt), t(step), n, C, width, True, True)
    gq = raymarch_backward(go, v, t(lab), t(M), t(src), t(tgt), t(step), n, C, width, True, True, quad=q)
    for a, b in zip(gp[1:], gq[1:]):  # gM, gsrc, gtgt, gstep
        assert rel_maxabs(b, a) < 1e-6
    assert rel_maxabs(gq[0], gp[0]) < 1e-5


def test_render_layout_choice_and_request(random32):
    """One pose without a gradient reads the plain volume (the quad copy's 4x
    bytes are not reused by other poses), several poses read the quad copy,
    and `subject.layout` overrides either; the images are the same."""
    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    k_inv, rt, sdd, H, W = rays_for(g)
    out_p = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200)
    assert getattr(sub, "_ndrr_quad_cache", None) is None
    out_q2 = nd.render(sub, k_inv, rt.expand(2, -1, -1), sdd, H, W, n_samples=200)
    assert getattr(sub, "_ndrr_quad_cache", None) is not None
    assert torch.equal(out_q2[:1], out_p) and torch.equal(out_q2[1:], out_p)
    sub.layout = "quad"
    out_q = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200)
    assert torch.equal(out_q, out_p)
    # the cached quad follows in-place volume edits
    sub._image_hu.mul_(2.0)
    out_2 = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=200)
    assert rel_maxabs(out_2, 2 * out_q) < 1e-6


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("C", [1, 4])
@pytest.mark.parametrize("seed", [41, 42])
def test_slab_ordered_adjoint_equals_direct(dtype, C, seed):
    """gvol_mode 3 (work ordered slab by slab across poses) marches every
    sample exactly once: the volume gradient agrees with the direct scatter
    to rounding, the pose gradient to fp32 regrouping (each ray's samples are
    split across slab items), and the pose gradient is bitwise reproducible.
    Random rotations exercise all three slab axes."""
    from nanodrr_gb300.raymarch import quad_volume

    n = 190
    vol, lab, M, src, tgt, step, width = _random_case(seed, B=4, Hd=22, Wd=26, vol_shape=(44, 38, 50), C=C)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol).to(dtype)
    q = quad_volume(v)
    go = torch.randn(4, C, 22 * 26, device=DEV)
    args = (go, v, t(lab), t(M), t(src), t(tgt), t(step), n, C, width, True, False)
    direct = raymarch_backward(*args, quad=q, gvol_mode=1)
    slab = raymarch_backward(*args, quad=q, gvol_mode=3)
    again = raymarch_backward(*args, quad=q, gvol_mode=3)
    assert rel_maxabs(slab[0], direct[0]) < 1e-5
    assert rel_maxabs(slab[1], direct[1]) < 1e-5
    assert torch.equal(slab[1], again[1])
    # gvol_mode 4: the same work with lanes that share a quad cell combining
    # their terms before the reduction; the pose gradient is untouched
    warp = raymarch_backward(*args, quad=q, gvol_mode=4)
    assert rel_maxabs(warp[0], direct[0]) < 1e-5
    assert torch.equal(warp[1], slab[1])
    if C == 1:  # (with labels, fp32-vs-fp64 label routing differs at label boundaries)
        ref = march_numpy_adjoint(go.double().cpu().numpy(), v.float().cpu().numpy().astype(np.float64), lab, M,
                                  src, tgt, step, n, C)
        assert rel_maxabs(slab[0], ref[0]) < 1e-4


@pytest.mark.parametrize("seed", [5, 6])
@pytest.mark.parametrize("accumulate", [False, True])
def test_thin_slabs_fold_their_boxes_exactly(seed, accumulate):
    """1 MiB slabs on a 96 x 80 x 88 volume: about 13 slabs per axis, so the
    scratch boxes are reused many times, every fold meets its neighbours'
    boundary planes and the two boxes alternate. The volume gradient equals
    the direct scatter (and accumulates onto a given gradient), the pose
    gradient is reproducible."""
    from nanodrr_gb300.raymarch import quad_volume

    n = 260
    vol, lab, M, src, tgt, step, width = _random_case(seed, B=6, Hd=20, Wd=24, vol_shape=(96, 80, 88), C=1)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol)
    q = quad_volume(v)
    go = torch.randn(6, 1, 20 * 24, device=DEV)
    args = (go, v, t(lab), t(M), t(src), t(tgt), t(step), n, 1, width, True, False)
    direct = raymarch_backward(*args, quad=q, gvol_mode=1)
    base = torch.randn_like(v) if accumulate else None
    gv = base.clone() if accumulate else None
    slab = raymarch_backward(*args, quad=q, gvol_mode=3, slab_mib=1, gvol=gv)
    again = raymarch_backward(*args, quad=q, gvol_mode=3, slab_mib=1)
    expect = direct[0] + base if accumulate else direct[0]
    assert rel_maxabs(slab[0], expect) < 1e-5
    assert rel_maxabs(slab[1], direct[1]) < 1e-5
    assert torch.equal(slab[1], again[1])
    assert torch.isfinite(slab[1]).all()


def test_slab_mode_needs_the_quad_layout():
    vol, lab, M, src, tgt, step, width = _random_case(43, B=1, Hd=8, Wd=8)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    go = torch.randn(1, 1, 64, device=DEV)
    with pytest.raises(ValueError, match="quad layout"):
        raymarch_backward(go, t(vol), t(vol), t(M), t(src), t(tgt), t(step), 100, 1, width, True, False, gvol_mode=3)


def test_texture_filtered_forward_variant_is_close():
    """The texture unit's trilinear filter (8-bit weights) against the fp32
    software path: close (about 1e-3 relative), not equal."""
    from nanodrr_gb300.raymarch import TextureVolume

    n = 220
    vol, lab, M, src, tgt, step, width = _random_case(51, B=2, Hd=24, Wd=20)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol)
    tex = TextureVolume(v)
    soft, _ = raymarch_forward(v, v, t(M), t(src), t(tgt), t(step), n, 1, width)
    hard, _ = raymarch_forward(v, v, t(M), t(src), t(tgt), t(step), n, 1, width, texture=tex)
    err = rel_maxabs(hard, soft)
    assert err < 1e-2, err
    assert float(hard.abs().max()) > 0
    tex.close()
    with pytest.raises(ValueError):
        raymarch_forward(v, v, t(M), t(src), t(tgt), t(step), n, 1, width, texture=tex)


@pytest.mark.parametrize("seed,vol_shape", [(61, (40, 36, 44)), (62, (70, 52, 64))])
def test_tma_staged_forward_variant_is_bitwise_the_default(seed, vol_shape):
    """The TMA variant gathers the same corners from shared-memory boxes (TMA
    zero fill outside the volume = zero padding) with the same arithmetic."""
    n = 230
    vol, lab, M, src, tgt, step, width = _random_case(seed, B=3, Hd=24, Wd=32, vol_shape=vol_shape)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol)
    ref, _ = raymarch_forward(v, v, t(M), t(src), t(tgt), t(step), n, 1, width, tile=(16, 8, 1))
    out, _ = raymarch_forward(v, v, t(M), t(src), t(tgt), t(step), n, 1, width, fwd_mode=1)
    assert torch.isfinite(out).all()
    assert torch.equal(out, ref)
    from nanodrr_gb300.raymarch import device_flags

    assert device_flags() & _ffi.NDRR_FLAG_TMA_TIMEOUT == 0  # no stage wait gave up


def test_rays_that_miss_the_volume_on_every_path():
    """Every ray passes beside the volume: zero images and gradients from the
    default, slab-ordered, TMA and texture paths (empty work lists, no chunk)."""
    from nanodrr_gb300.raymarch import TextureVolume, quad_volume

    n = 120
    vol, lab, M, src, tgt, step, width = _random_case(71, B=2, Hd=16, Wd=16, vol_shape=(24, 20, 28))
    M = M.copy()
    M[:, :, 3] += 1000.0  # shift every ray far outside the box
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol)
    q = quad_volume(v)
    args = (v, v, t(M), t(src), t(tgt), t(step), n, 1, width)
    out, _ = raymarch_forward(*args, quad=q)
    assert float(out.abs().max()) == 0.0
    tma, _ = raymarch_forward(*args, fwd_mode=1)
    assert float(tma.abs().max()) == 0.0
    tex = TextureVolume(v)
    hard, _ = raymarch_forward(*args, texture=tex)
    tex.close()
    assert float(hard.abs().max()) == 0.0
    go = torch.ones_like(out)
    gvol, gM, *_ = raymarch_backward(go, *args, True, False, quad=q, gvol_mode=3)
    assert float(gvol.abs().max()) == 0.0 and float(gM.abs().max()) == 0.0


def test_quad_adjoint_accumulates_into_a_given_gradient():
    """With a caller's gvol the adjoint adds (two calls give twice one call);
    with none it writes a fresh one (no zeroing pass)."""
    from nanodrr_gb300.raymarch import quad_volume

    n = 150
    vol, lab, M, src, tgt, step, width = _random_case(72, B=2, Hd=18, Wd=20)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol)
    q = quad_volume(v)
    go = torch.randn(2, 1, 18 * 20, device=DEV)
    args = (go, v, v, t(M), t(src), t(tgt), t(step), n, 1, width, True, False)
    fresh = raymarch_backward(*args, quad=q)[0]
    acc = torch.zeros_like(v)
    raymarch_backward(*args, quad=q, gvol=acc)
    raymarch_backward(*args, quad=q, gvol=acc)
    assert rel_maxabs(acc, 2 * fresh) < 1e-5


def test_ray_cache_follows_the_camera_tensors(random32):
    """Repeated renders reuse the ray set-up of the same k_inv / sdd tensors;
    an in-place change of either, or a new tensor, gives the uncached result;
    a recorded gradient and the no-gradient direct call agree bitwise."""
    from nanodrr_gb300 import renderer

    g = random32
    sub = subject_from_arrays(g["vol"], None, g["voxel_to_world"], 1)
    k_inv, rt, sdd, H, W = rays_for(g)
    n = int(g["n_samples"])

    def fresh(k, s):  # cache bypassed: explicit rays
        tgt = renderer._make_tgt(k, s, H, W, rt.device, rt.dtype)
        src = renderer._make_src(False, tgt, s)
        return nd.render(sub, k, rt, s, H, W, n_samples=n, src=src, tgt=tgt)

    with torch.no_grad():
        a = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=n)
        b = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=n)
        assert torch.equal(a, b)
        assert torch.equal(a, fresh(k_inv, sdd))
        k_inv[..., 0, 0] *= 1.1  # in place: the version counter moves
        c = nd.render(sub, k_inv, rt, sdd, H, W, n_samples=n)
        assert not torch.equal(c, a)
        assert torch.equal(c, fresh(k_inv, sdd))
        s2 = sdd * 0.9  # a new tensor
        d = nd.render(sub, k_inv, rt, s2, H, W, n_samples=n)
        assert torch.equal(d, fresh(k_inv, s2))
    rg = rt.clone().requires_grad_(True)
    e = nd.render(sub, k_inv, rg, sdd, H, W, n_samples=n)
    assert torch.equal(e.detach(), c)


@pytest.mark.parametrize("axis_dir", [(0.3, 0.1, 0.95), (0.1, 0.3, 0.95), (0.1, 0.95, 0.3), (0.95, 0.2, 0.1)])
def test_slab_axis_choices_equal_direct(axis_dir):
    """Optical axes chosen so that each slab axis is used (rays mostly along z
    give y or x slabs, others z slabs), with 1 MiB slabs: volume and pose
    gradients equal the direct scatter."""
    from nanodrr_gb300.raymarch import quad_volume

    vol, lab, M, src, tgt, step, width = _random_case(11, B=2, Hd=20, Wd=24, vol_shape=(72, 64, 80), C=1)
    d = np.array(axis_dir, np.float64)
    d /= np.linalg.norm(d)
    a = np.cross(d, [0.0, 0.0, 1.0] if abs(d[2]) < 0.9 else [1.0, 0.0, 0.0])
    a /= np.linalg.norm(a)
    R = np.stack([a, np.cross(d, a), d], 1)  # columns: detector u, v and the optical axis
    for b in range(2):
        M[b, :, :3] = (R * (1.0 + 0.1 * b)).astype(np.float32)
    t = lambda x: torch.from_numpy(x).to(DEV)  # noqa: E731
    v = t(vol)
    q = quad_volume(v)
    go = torch.randn(2, 1, 20 * 24, device=DEV)
    args = (go, v, t(lab), t(M), t(src), t(tgt), t(step), 240, 1, width, True, False)
    direct = raymarch_backward(*args, quad=q, gvol_mode=1)
    slab = raymarch_backward(*args, quad=q, gvol_mode=3, slab_mib=1)
    assert rel_maxabs(slab[0], direct[0]) < 1e-5
    assert rel_maxabs(slab[1], direct[1]) < 1e-5


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float16])
@pytest.mark.parametrize("lab_dtype", [torch.uint8, torch.float32])
def test_labelled_quad_equals_quad_with_label_gathers(dtype, lab_dtype):
    """The labelled quad layout carries each corner's class in the 16-byte
    element: the per-label forward (with the total) is bitwise the plain quad
    layout's with label gathers, the adjoint's pose gradient bitwise, its
    volume gradient to atomics rounding — through the direct and the
    slab-ordered adjoints, with the out-of-range class value dropped and
    rays that leave the volume."""
    from nanodrr_gb300.raymarch import quad_volume, quad_volume_labeled

    n, C = 190, 5
    vol, lab, M, src, tgt, step, width = _random_case(83, B=3, Hd=20, Wd=24, vol_shape=(40, 36, 44), C=C)
    t = lambda a: torch.from_numpy(a).to(DEV)  # noqa: E731
    v = t(vol).to(dtype)
    lb = t(lab).to(lab_dtype)
    q = quad_volume(v)
    ql = quad_volume_labeled(v, lb, C)
    assert ql.numel() == 2 * q.numel()
    args = (v, lb, t(M), t(src), t(tgt), t(step), n, C, width)
    ref, ref_total = raymarch_forward(*args, quad=q, with_total=True)
    out, total = raymarch_forward(*args, quad=ql, with_total=True)
    assert torch.equal(out, ref) and torch.equal(total, ref_total)
    assert float(out.float().abs().max()) > 0
    go = torch.randn(3, C, 20 * 24, device=DEV)
    for mode, gcam in ((1, True), (3, False)):
        bargs = (go, *args, True, gcam)
        a = raymarch_backward(*bargs, quad=q, gvol_mode=mode)
        b = raymarch_backward(*bargs, quad=ql, gvol_mode=mode)
        assert torch.equal(a[1], b[1])
        assert rel_maxabs(b[0], a[0]) < 1e-5
        if gcam:
            for ga, gb in zip(a[2:], b[2:]):
                assert torch.equal(ga, gb)


def test_labelled_quad_is_the_render_path_for_16_bit_per_label_volumes():
    """render() of a bf16 subject with labels reads the labelled quad, and its
    image equals the plain-layout render's."""
    from nanodrr_gb300 import phantom
    from nanodrr_gb300.renderer import cached_quad, compact_label

    ph = phantom.make_phantom((40, 40, 40), (128 / 40,) * 3, seed=4)
    sub = ph.subject(dtype=torch.bfloat16, with_labels=True, device=DEV)
    k_inv, sdd = phantom.detector(pixel=1.4 * 200 / 32, height=32, width=32)
    rt = phantom.random_poses(2, seed=9).to(DEV)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    with torch.no_grad():
        out = nd.render(sub, k_inv, rt, sdd, 32, 32, n_samples=300)
        vol = sub.image[0, 0]
        q = cached_quad(sub, vol, compact_label(sub), sub.n_classes)
        assert q.numel() == (40 + 4) * 43 * 43 * 16  # labelled elements
        sub.layout = "plain"
        plain = nd.render(sub, k_inv, rt, sdd, 32, 32, n_samples=300)
    assert rel_maxabs(out.float(), plain.float()) < 1e-2  # bf16 output rounding of fp32 sums
    assert torch.equal(out.float().sum(1).abs() > 0, plain.float().sum(1).abs() > 0)


def test_measurement_probes_run_and_count():
    """The library's probes behind the bench's roofline: the reduction probe
    adds 1.0 to four floats of two quad entries per thread and iteration
    (the total is exact), the L2 read probe and the kernel-event hook run
    without touching results."""
    lib = _ffi.load()
    buf = torch.zeros(6 * 512 * 512 * 4, dtype=torch.float32, device=DEV)  # 6 planes of quad entries
    n = ctypes.c_int32(0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.ndrr_reduce_probe(ctypes.c_void_p(buf.data_ptr()), ctypes.c_uint64(buf.numel() * 4), 3, ctypes.byref(n),
                               ctypes.c_void_p(stream))
    assert rc == _ffi.NDRR_OK
    torch.cuda.synchronize()
    assert n.value > 0 and float(buf.double().sum()) == n.value * 3 * 2 * 4
    sink = torch.zeros(1, dtype=torch.int32, device=DEV)
    src = torch.ones(1 << 20, dtype=torch.uint8, device=DEV)
    assert lib.ndrr_l2_read_probe(ctypes.c_void_p(src.data_ptr()), ctypes.c_uint64(src.numel()), 2,
                                  ctypes.c_void_p(sink.data_ptr()), ctypes.c_void_p(stream)) == _ffi.NDRR_OK
    torch.cuda.synchronize()
    assert int(sink.item()) == 0
