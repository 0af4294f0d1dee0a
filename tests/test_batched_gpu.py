"""Persistent batched launch: every request of a heterogeneous batch (three
volumes, mixed detector sizes and sample counts) gets exactly what the
single-request kernels give with the same launch shape, the pose adjoint
included; a CUDA graph of the whole step replays with new poses; the
autotuner picks a valid shape and caches it."""

import numpy as np
import pytest
import torch

from nanodrr_gb300 import phantom
from nanodrr_gb300.autotune import BATCHED_CANDIDATES, Autotuner
from nanodrr_gb300.batched import BatchedRenderer, RenderRequest
from nanodrr_gb300.raymarch import raymarch_backward, raymarch_forward

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _requests(n=9, C=1, seed=0):
    vols = [
        phantom.make_phantom((24, 24, 24), (6.0, 6.0, 6.0), seed=1).subject(device=DEV, with_labels=C > 1),
        phantom.make_phantom((20, 32, 28), (4.0, 4.0, 6.0), seed=2).subject(device=DEV, with_labels=C > 1),
        phantom.make_phantom((36, 18, 18), (5.0, 5.0, 3.0), seed=3).subject(device=DEV, with_labels=C > 1),
    ]
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        det = int(rng.choice([12, 16, 20, 24, 33]))
        k_inv, sdd = phantom.detector(pixel=300.0 / det, height=det, width=det)
        reqs.append(RenderRequest(vols[i % 3], k_inv.to(DEV), sdd.to(DEV), det, det, int(rng.integers(30, 100))))
    poses = phantom.random_poses(n, seed=seed + 11).to(DEV)
    return reqs, poses


@pytest.mark.parametrize("layout", ["quad", "plain"])
@pytest.mark.parametrize("C", [1, 8])
def test_batched_matches_single_requests(C, layout):
    reqs, poses = _requests(C=C)
    br = BatchedRenderer(reqs, n_classes=C, layout=layout)
    br.set_poses(poses)
    br.forward()
    for i, r in enumerate(reqs):
        shape = br.shapes[i]
        vol = br.vols[i]
        M = br.M[i : i + 1]
        out, _ = raymarch_forward(vol, br.labs[i], M, br.src[i], br.tgt[i], br.step[i], r.n_samples, C, r.width,
                                  tile=shape, quad=br.quads[i])
        assert torch.equal(br.output(i).reshape(out.shape), out), i
        if layout == "quad":  # the quad layout holds exact copies: the plain march's image too
            plain, _ = raymarch_forward(vol, br.labs[i], M, br.src[i], br.tgt[i], br.step[i], r.n_samples, C,
                                        r.width, tile=shape)
            assert torch.equal(plain, out), i
    # pose adjoint
    for i in range(len(reqs)):
        br.go(i).copy_(torch.randn_like(br.go(i)))
    br.backward()
    for i, r in enumerate(reqs):
        go = br.go(i).reshape(1, C, -1)
        _, gM, *_ = raymarch_backward(go, br.vols[i], br.labs[i], br.M[i : i + 1], br.src[i], br.tgt[i],
                                      br.step[i], r.n_samples, C, r.width, False, False, tile=br.shapes[i],
                                      quad=br.quads[i])
        assert torch.equal(br.gM[i], gM[0]), i


def test_batched_step_replays_in_a_cuda_graph():
    reqs, poses = _requests(n=6, seed=3)
    br = BatchedRenderer(reqs)
    w = [torch.randn_like(br.output(i)) for i in range(len(reqs))]
    pose_in = poses.clone()

    def step():
        br.set_poses(pose_in)
        br.forward()
        for i in range(len(reqs)):
            br.go(i).copy_(w[i])
        br.backward()

    step()  # warm-up (loads the library, first-launch attributes)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    new = phantom.random_poses(len(reqs), seed=77).to(DEV)
    pose_in.copy_(new)
    g.replay()
    torch.cuda.synchronize()
    graph_out = [br.output(i).clone() for i in range(len(reqs))]
    graph_gM = br.gM.clone()
    step()  # eager with the same poses
    torch.cuda.synchronize()
    for i in range(len(reqs)):
        assert torch.equal(graph_out[i], br.output(i))
    assert torch.equal(graph_gM, br.gM)


def test_autotuner_picks_and_caches_a_valid_shape(tmp_path):
    reqs, poses = _requests(n=3)
    tuner = Autotuner(tmp_path / "tune.json", reps=2)
    br = BatchedRenderer(reqs, autotuner=tuner)
    assert all(s in BATCHED_CANDIDATES for s in br.shapes)
    assert (tmp_path / "tune.json").exists()
    again = Autotuner(tmp_path / "tune.json")
    assert len(again.cache) >= 1


def test_autotuner_picks_a_slab_size_and_render_uses_it(tmp_path):
    import nanodrr_gb300 as nd
    from nanodrr_gb300.autotune import SLAB_CANDIDATES
    from nanodrr_gb300.raymarch import quad_volume
    from nanodrr_gb300.renderer import _affine_product, _make_src, _make_tgt

    sub = phantom.make_phantom((40, 36, 44), (3.0, 3.0, 3.0), seed=4).subject(device=DEV)
    vol = sub.image[0, 0].contiguous()
    k_inv, sdd = phantom.detector(pixel=4.0, height=24, width=24)
    k_inv, sdd = k_inv.to(DEV), sdd.to(DEV)
    rt = phantom.random_poses(3, seed=6).to(DEV)
    tgt = _make_tgt(k_inv, sdd, 24, 24, DEV, torch.float32).expand(3, -1, -1).contiguous()
    src = _make_src(False, tgt, sdd.expand(3)).contiguous()
    step = ((tgt - src).norm(dim=-1) / 149).contiguous()
    M = _affine_product(sub.world_to_voxel[:3], rt).contiguous()
    tuner = Autotuner(tmp_path / "tune.json", reps=2)
    # tiny slabs (1 MiB) so that the work splits across many slabs here
    mib = tuner.best_slab_mib(vol, quad_volume(vol), M, src, tgt, step, 150, 24, candidates=[1, 2, 96])
    assert mib in (1, 2, 96)
    assert Autotuner(tmp_path / "tune.json").best_slab_mib(vol, None, M, src, tgt, step, 150, 24,
                                                           candidates=[1, 2, 96]) == mib  # cached
    assert SLAB_CANDIDATES
    # render with a volume gradient: slab size 1 MiB equals the default
    vol_param = sub._image_hu.detach().clone().requires_grad_(True)
    sub._image_hu = vol_param
    w = torch.randn(3, 1, 24, 24, device=DEV)
    (nd.render(sub, k_inv, rt, sdd, 24, 24, n_samples=150) * w).sum().backward()
    g_default = vol_param.grad.clone()
    vol_param.grad = None
    sub.slab_mib = 1
    (nd.render(sub, k_inv, rt, sdd, 24, 24, n_samples=150) * w).sum().backward()
    rel = float((vol_param.grad - g_default).abs().max() / g_default.abs().max())
    assert rel < 1e-5
