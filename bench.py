#!/usr/bin/env python
"""Benchmark: forward + backward DRR frames/s on one GB300.

Workload (one "step" = one batch of poses through the render and its adjoint):
a registration step on the seeded CT phantom — 512 x 512 x 512 float32
volume (0.8 x 0.8 x 1.0 mm voxels), 32 poses (ZXY rotations uniform ±30°,
translations ±50 mm about a source 600 mm from the isocenter), 256 x 256
detector at 1.2 mm, SDD 1020 mm, 800 samples per ray; loss = NCC against
target DRRs rendered at held-out poses; backward to the se(3) 6-vector of
every pose and to the volume. One frame = one pose's image forward + backward.

Arms:
  default           the CUDA kernels (this package);
  --impl reference  the reference's CPU path (its PyTorch grid_sample backend,
                    restated in oracle/) on the host cores, on a bounded
                    sample of the same workload.

Prints one JSON line (rank 0). Under torchrun every rank renders its own
pose batch against its own copy of the volume (no collective on the data
path; weak scaling); the timed region is bracketed by barriers and the max
over ranks is reported.
"""

from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import torch  # noqa: E402

BASELINE_HEADLINE = None  # no published number exists for this metric
METRIC = "fwd+bwd DRR frames/s at 512^3/256^2, learned-skip vs plain kernel"
# DRAM read + write bytes per sample of the slab-ordered adjoint kernel,
# measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum of one launch)
# on a 384^3 x 8-pose case of the same kernel and scaled here by the samples
# of a launch.
SLAB_DRAM_BYTES_PER_SAMPLE = 19.67
SLAB_DRAM_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, 384^3 x 8 poses, scaled per sample"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--volume", default="512x512x512", help="DxHxW voxels")
    p.add_argument("--spacing", default="0.8,0.8,1.0", help="sx,sy,sz mm")
    p.add_argument("--batch", type=int, default=32)
    p.add_argument("--det", type=int, default=256)
    p.add_argument("--pixel", type=float, default=1.2)
    p.add_argument("--samples", type=int, default=800)
    p.add_argument("--cpu-rays", type=int, default=2048, help="rays per CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--method", default="learned", choices=["plain", "occupancy", "learned"])
    p.add_argument("--train-poses", type=int, default=16)
    p.add_argument("--prop-epochs", type=int, default=40)
    p.add_argument("--no-batched", action="store_true", help="skip the uneven batched-launch measurement")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the per-label forward and the 1024^2 learned-proposal measurements")
    p.add_argument("--no-reference-kernel", action="store_true",
                   help="skip timing the reference's Triton kernel from baseline/_ref")
    p.add_argument("--no-graph", action="store_true",
                   help="time eager steps only (no CUDA-graph capture; for profilers that cannot follow a capture)")
    return p.parse_args()


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi clock/throttle sampling in the background (200 ms)."""

    FIELDS = (
        "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
        "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
        "clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.index)],
                stdout=self.file, stderr=subprocess.DEVNULL,
            )
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.count(",") >= 6]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                smax = float(r[1])
            except ValueError:
                continue
            for name, v in zip(names, r[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        load = [s for s in sm if smax and s > 0.5 * smax] or sm
        return {
            "sm_mhz": statistics.median(load) if load else None,
            "sm_max_mhz": smax,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch.distributed as dist

    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def parse_shape(s):
    return tuple(int(v) for v in s.lower().split("x"))


def workload(args, device, seed_offset=0):
    """Phantom subject, detector, base poses, perturbation pivots and targets."""
    from nanodrr_gb300 import phantom

    D, H, W = parse_shape(args.volume)
    sp = tuple(float(v) for v in args.spacing.split(","))
    gen_dev = device if torch.cuda.is_available() else "cpu"
    ph = phantom.make_phantom((D, H, W), sp, seed=0, device=gen_dev)
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=args.pixel, height=args.det, width=args.det)
    rt = phantom.random_poses(args.batch, seed=1 + seed_offset)
    # held-out targets: the same poses perturbed by up to 0.05 rad / 5 mm
    held = _nudge(rt, seed=77 + seed_offset)
    return ph, k_inv, sdd, rt, held


def _nudge(rt, seed):
    from nanodrr_gb300.geometry import convert

    g = torch.Generator().manual_seed(seed)
    rot = (torch.rand(rt.shape[0], 3, generator=g) * 2 - 1) * 0.05
    xyz = (torch.rand(rt.shape[0], 3, generator=g) * 2 - 1) * 5.0
    return rt @ convert(rot, xyz, "so3_log")


# --------------------------------------------------------------- our arm
def count_samples(M, src, tgt, D, H, W, S):
    """Samples inside each ray's march window (same rule as the kernel)."""
    p0 = torch.einsum("bij,bnj->bni", M[:, :, :3], src.expand_as(tgt)) + M[:, None, :, 3]
    d = torch.einsum("bij,bnj->bni", M[:, :, :3], tgt - src)
    lo_b = torch.tensor([-2.0, -2.0, -2.0], device=M.device)
    hi_b = torch.tensor([W + 1.0, H + 1.0, D + 1.0], device=M.device)
    dd = torch.where(d.abs() < 1e-20, torch.full_like(d, 1e-20), d)
    a = (lo_b - p0) / dd
    b = (hi_b - p0) / dd
    t_lo = torch.minimum(a, b).amax(-1)
    t_hi = torch.maximum(a, b).amin(-1)
    f_lo = (torch.floor(t_lo * (S - 1)) - 2).clamp(0, S)
    f_hi = (torch.ceil(t_hi * (S - 1)) + 3).clamp(0, S)
    n = (f_hi - f_lo).clamp(min=0)
    n = torch.where(t_lo <= t_hi, n, torch.zeros_like(n))
    return float(n.sum())


def warp_cell_sharing(M, src, tgt, D, H, W, S, det, poses=4, warps=512, seed=0):
    """Lanes per distinct cell among the 32 rays of a warp (8 x 4 detector
    pixels, the kernels' warp shape) at each iteration of the adjoint's
    sample loop, where a lane's sample is its ray's first windowed sample
    plus the iteration (the window rule of count_samples), over a seeded
    subset of warps: how many of a warp's reductions could merge into one
    per cell (warp-aggregated atomics)."""
    dev = M.device
    g = torch.Generator().manual_seed(seed)
    n_wx, n_wy = det // 8, det // 4
    lane = torch.arange(32)
    lanes = cells = 0
    for b in range(min(poses, M.shape[0])):
        wid = torch.randperm(n_wx * n_wy, generator=g)[:warps]
        px = (wid % n_wx)[:, None] * 8 + lane % 8
        py = (wid // n_wx)[:, None] * 4 + lane // 8
        n = (py * det + px).reshape(-1).to(dev)
        Mb = M[b].double()
        s_b = src[b].double().expand(tgt.shape[1], -1)[n]
        d_cam = tgt[b].double()[n] - s_b
        p0 = s_b @ Mb[:, :3].T + Mb[:, 3]
        d = d_cam @ Mb[:, :3].T
        lo_b = torch.tensor([-2.0, -2.0, -2.0], device=dev, dtype=torch.float64)
        hi_b = torch.tensor([W + 1.0, H + 1.0, D + 1.0], device=dev, dtype=torch.float64)
        dd = torch.where(d.abs() < 1e-20, torch.full_like(d, 1e-20), d)
        ta, tb = (lo_b - p0) / dd, (hi_b - p0) / dd
        t_lo, t_hi = torch.minimum(ta, tb).amax(-1), torch.maximum(ta, tb).amin(-1)
        f_lo = (torch.floor(t_lo * (S - 1)) - 2).clamp(0, S)
        f_hi = (torch.ceil(t_hi * (S - 1)) + 3).clamp(0, S)
        f_hi = torch.where(t_lo <= t_hi, f_hi, f_lo)
        it = torch.arange(S, device=dev, dtype=torch.float64)
        s_idx = f_lo[:, None] + it[None, :]  # [rays, iterations]
        active = s_idx < f_hi[:, None]
        pos = p0[:, None, :] + (s_idx / (S - 1))[..., None] * d[:, None, :]
        ix = torch.floor(pos).clamp(min=-2).long()
        ix = torch.minimum(ix, torch.tensor([W, H, D], device=dev))
        cid = ((ix[..., 2] + 2) * (H + 3) + (ix[..., 1] + 2)) * (W + 3) + (ix[..., 0] + 2)
        # inactive lanes get distinct negative ids, then distinct = sorted runs
        cid = torch.where(active, cid, -1 - torch.arange(cid.numel(), device=dev).reshape(cid.shape))
        cid = cid.reshape(-1, 32, S).transpose(1, 2)  # [warps, iterations, lanes]
        act = active.reshape(-1, 32, S).transpose(1, 2)
        srt = cid.sort(dim=-1).values
        new = torch.ones_like(srt, dtype=torch.bool)
        new[..., 1:] = srt[..., 1:] != srt[..., :-1]
        srt_act = srt >= 0
        lanes += int(act.sum())
        cells += int((new & srt_act).sum())
    return lanes / max(cells, 1)


def run_ours(args, world, rank, local):
    import nanodrr_gb300 as nd
    from nanodrr_gb300 import _build
    from nanodrr_gb300.empty_space import EmptySpace, train_proposal
    from nanodrr_gb300.raymarch import raymarch_backward, raymarch_forward, skip_windows
    from nanodrr_gb300.registration import GraphedStep, NormalizedCrossCorrelation2d, Registration
    from nanodrr_gb300.renderer import _affine_product, _make_src, _make_tgt, cached_quad

    _build.build()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ph, k_inv, sdd, rt, held = workload(args, dev, seed_offset=rank)
    sub = ph.subject(device=dev)
    del ph
    vol_param = sub._image_hu.detach().requires_grad_(True)
    sub._image_hu = vol_param
    vol = vol_param.detach()[0, 0]
    D, H, W = vol.shape
    k_inv, sdd, rt, held = k_inv.to(dev), sdd.to(dev), rt.to(dev), held.to(dev)
    B, Hd, S = args.batch, args.det, args.samples
    with torch.no_grad():
        target = nd.render(sub, k_inv, held, sdd, Hd, Hd, n_samples=S)
    ncc = NormalizedCrossCorrelation2d()
    reg = Registration(sub, rt, k_inv, sdd, Hd, Hd, batch=B).to(dev)
    tgt = _make_tgt(k_inv, sdd, Hd, Hd, dev, torch.float32)
    src = _make_src(False, tgt, sdd)

    # ---- learned proposal: labels from the plain renderer on training poses
    # (a seed disjoint from the benchmark poses), fitted by the project's
    # training kernels; then the occupancy grid that checks it.
    from nanodrr_gb300 import phantom

    t0 = time.perf_counter()
    rt_train = phantom.random_poses(args.train_poses, seed=500 + rank).to(dev)
    Mt = _affine_product(sub.world_to_voxel[:3], rt_train).contiguous()
    tgt_t = tgt.expand(args.train_poses, -1, -1).contiguous()
    src_t = src.expand(args.train_poses, -1, -1).contiguous()
    step_t = ((tgt_t - src_t).norm(dim=-1) / (S - 1)).contiguous()
    net, hist = train_proposal(vol, Mt, src_t, tgt_t, step_t, S, Hd, epochs=args.prop_epochs, batch=65536,
                               lr=2e-3, alpha=20.0)
    skips = {
        "plain": None,
        "occupancy": EmptySpace.occupancy(vol, cell=4),
        "learned": EmptySpace.proposal(vol, net, cell=4, margin=2.0),
    }
    torch.cuda.synchronize()
    prep_s = time.perf_counter() - t0

    def make_step(skip, vol_grad):
        def step():
            sub.empty_space = skip
            vol_param.grad = None
            reg._rot.grad = None
            reg._xyz.grad = None
            sub._image_hu = vol_param if vol_grad else vol_param.detach()
            img = reg(n_samples=S)
            loss = -ncc(img, target).mean()
            loss.backward()
            return loss

        return step

    def timed(fn, steps):
        for _ in range(max(args.warmup, 3)):
            fn()
        barrier(world)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        barrier(world)
        return max_over_ranks(e0.elapsed_time(e1) / 1e3, world, dev)

    def graphed(skip, vol_grad):
        """The same step captured in a CUDA graph (GraphedStep)."""
        sub.empty_space = skip
        sub._image_hu = vol_param if vol_grad else vol_param.detach()
        return GraphedStep(reg, lambda img, tgt_img: -ncc(img, tgt_img).mean(), target, n_samples=S)

    headline = args.method
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    table, eager = {}, {}
    for name, skip in skips.items():
        for vg in (True, False):
            key = f"{name}{'' if vg else '_pose_only'}"
            t = timed(make_step(skip, vg), args.steps)
            eager[key] = round(B * args.steps * world / t, 2)
            if not args.no_graph:
                t = timed(graphed(skip, vg).replay, args.steps)
            table[key] = round(B * args.steps * world / t, 2)
    # headline last, with the clocks still sampling; its warm-up and timed
    # steps sit between cudaProfilerStart/Stop, so a profiler started with
    # collection off (ncu --profile-from-start off) records their launches only
    if args.no_graph:
        head_step = None
        torch.cuda.profiler.start()
        t_dev = timed(make_step(skips[headline], True), args.steps)
    else:
        head_step = graphed(skips[headline], True)
        torch.cuda.profiler.start()
        t_dev = timed(head_step.replay, args.steps)
    torch.cuda.profiler.stop()
    clk = clocks.stop()
    frames = B * args.steps * world
    value = frames / t_dev

    # ---- end to end through the public API: per step the pose 6-vectors
    # come from pinned host memory into the graph's static parameters and the
    # loss + pose gradients go back to pinned host memory.
    host_params = torch.zeros(B, 6, pin_memory=True)
    host_out = torch.zeros(1 + B * 6, pin_memory=True)
    eager_step = make_step(skips[headline], True)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.no_grad():
            p = host_params.to(dev, non_blocking=True)
            reg._rot.copy_(p[:, :3])
            reg._xyz.copy_(p[:, 3:])
        if head_step is not None:
            loss = head_step.replay()
            g_rot, g_xyz = head_step.grads[0], head_step.grads[1]
        else:
            loss = eager_step().detach()
            g_rot, g_xyz = reg._rot.grad, reg._xyz.grad
        res = torch.cat([loss[None], g_rot.flatten(), g_xyz.flatten()])
        host_out.copy_(res, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world, dev)
    barrier(world)
    e2e = {
        "value": round(frames / t_e2e, 2),
        "unit": "frames/s",
        "h2d_bytes_per_step": host_params.numel() * 4,
        "d2h_bytes_per_step": host_out.numel() * 4,
    }

    # ---- per-kernel timing for the roofline, on the launch stream
    with torch.no_grad():
        pose = reg.pose.detach()
        M = _affine_product(sub.world_to_voxel[:3], pose).contiguous()
        tgtb = tgt.expand(B, -1, -1).contiguous()
        srcb = src.expand(B, -1, -1).contiguous()
        stepsz = ((tgtb - srcb).norm(dim=-1) / (S - 1)).contiguous()
        go = torch.randn(B, 1, Hd * Hd, device=dev)
        n_samp = count_samples(M, srcb, tgtb, D, H, W, S)
        stats = torch.zeros(4, dtype=torch.int64, device=dev)
        raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, skip=skips["learned"], stats=stats)
        occ_stats = torch.zeros(4, dtype=torch.int64, device=dev)
        raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, skip=skips["occupancy"], stats=occ_stats)
        gvol = torch.zeros_like(vol)
        quad = cached_quad(sub, vol)
        reps = max(3, args.steps)
        bwd_kernel_ms = _kernel_only_ms(
            lambda: raymarch_backward(go, vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, True, False, gvol=gvol,
                                      quad=quad), reps)
        fwd_kernel_ms = _kernel_only_ms(lambda: raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd,
                                                                 quad=quad), reps)
        l2 = l2_read_peak(dev)
        red = reduction_peak(dev)
        times = {"fwd": [], "fwd_learned": [], "bwd": [], "fwd_plain_layout": [], "bwd_plain_layout": [],
                 "learned_windows": [], "bwd_direct": []}
        for i in range(reps + 1):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(9)]
            e[0].record()
            raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, quad=quad)
            e[1].record()
            raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, skip=skips["learned"], quad=quad)
            e[2].record()
            # the step's adjoint: pose + volume gradient (slab-ordered, quad layout)
            raymarch_backward(go, vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, True, False, gvol=gvol, quad=quad)
            e[3].record()
            raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd)
            e[4].record()
            raymarch_backward(go, vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, True, False, gvol=gvol)
            e[5].record()
            skip_windows(vol, M, srcb, tgtb, stepsz, S, Hd, skips["learned"])
            e[6].record()
            raymarch_backward(go, vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, True, False, gvol=gvol, quad=quad,
                              gvol_mode=1)
            e[7].record()
            torch.cuda.synchronize()
            if i > 0:
                times["fwd"].append(e[0].elapsed_time(e[1]))
                times["fwd_learned"].append(e[1].elapsed_time(e[2]))
                times["bwd"].append(e[2].elapsed_time(e[3]))
                times["fwd_plain_layout"].append(e[3].elapsed_time(e[4]))
                times["bwd_plain_layout"].append(e[4].elapsed_time(e[5]))
                times["learned_windows"].append(e[5].elapsed_time(e[6]))
                times["bwd_direct"].append(e[6].elapsed_time(e[7]))
    e_bytes = vol.element_size()
    fwd_bytes = n_samp * 8 * e_bytes
    bwd_bytes = n_samp * (8 * e_bytes + 4 + 8 * 4 * 2)
    fwd_s = statistics.median(times["fwd"]) / 1e3
    bwd_s = statistics.median(times["bwd"]) / 1e3
    fwdl_s = statistics.median(times["fwd_learned"]) / 1e3
    kern_s = bwd_kernel_ms / 1e3
    peaks = _peaks()
    traffic = SLAB_DRAM_BYTES_PER_SAMPLE * n_samp
    dram_gbs = traffic / kern_s / 1e9
    demand_gbs = bwd_bytes / kern_s / 1e9
    st = stats.tolist()
    ost = occ_stats.tolist()
    roofline = {
        "bound": "hbm",
        "kernel": "raymarch_bwd_slab_kernel (adjoint with pose and volume gradient, slab-ordered, quad layout)",
        "timed": "the march kernel alone (CUDA events the library records around it on the launch stream)",
        # DRAM bytes of one launch per kernel time, against the measured HBM
        # copy bandwidth: the fraction of HBM the kernel uses
        "achieved": round(dram_gbs, 1),
        "peak": peaks["hbm_gbs"],
        "peak_source": peaks["source"],
        "unit": "GB/s",
        "frac": round(dram_gbs / peaks["hbm_gbs"], 4),
        "traffic": round(traffic, 1),
        "traffic_source": SLAB_DRAM_SOURCE,
        # the per-sample demand bytes (8 corner reads, the upstream gradient,
        # 8 corner read-modify-writes), mostly served by L1 and L2, against the
        # L2 read bandwidth measured by the library's probe in this run
        "algorithmic_bytes_per_launch": bwd_bytes,
        "demand_gbs": round(demand_gbs, 1),
        "l2_peak_gbs": l2["gbs"],
        "l2_peak_how": l2["how"],
        "l2_frac": round(demand_gbs / l2["gbs"], 4) if l2["gbs"] else None,
        "samples_per_launch": n_samp,
        "kernel_ms": round(bwd_kernel_ms, 3),
        "call_ms": round(bwd_s * 1e3, 3),
        "fwd_kernel_ms": round(fwd_kernel_ms, 3),
        "fwd_ms": round(fwd_s * 1e3, 3),
        "fwd_learned_ms": round(fwdl_s * 1e3, 3),
        "learned_windows_ms": round(statistics.median(times["learned_windows"]), 3),
        "fwd_gsamples_per_s": round(n_samp / fwd_s / 1e9, 2),
        "bwd_gsamples_per_s": round(n_samp / kern_s / 1e9, 2),
        # the scatter's two 16-byte reductions per sample alone, into an
        # L2-resident array (library probe, this run): the ceiling the
        # adjoint's sample rate is bound by
        "reduction_peak_gsamples_per_s": red["gsamples_per_s"],
        "reduction_peak_how": red["how"],
        "reduction_frac": round(n_samp / kern_s / 1e9 / red["gsamples_per_s"], 4) if red["gsamples_per_s"] else None,
        "fwd_demand_l2_frac": round(fwd_bytes / (fwd_kernel_ms / 1e3) / 1e9 / l2["gbs"], 4) if l2["gbs"] else None,
        "plain_layout_fwd_ms": round(statistics.median(times["fwd_plain_layout"]), 3),
        "plain_layout_bwd_ms": round(statistics.median(times["bwd_plain_layout"]), 3),
        "direct_scatter_bwd_ms": round(statistics.median(times["bwd_direct"]), 3),
    }
    # ---- warp-aggregated reductions: the sharing they can exploit, and the
    # slab kernel with them (gvol_mode 4) against the default, kernel alone
    with torch.no_grad():
        warp_agg = {
            "lanes_per_cell": round(warp_cell_sharing(M, srcb, tgtb, D, H, W, S, Hd), 3),
            "how": "32 rays of a warp (8 x 4 pixels) per loop iteration, lane sample = window start + "
                   "iteration, 512 seeded warps of each of 4 poses",
            "slab_kernel_ms": round(bwd_kernel_ms, 3),
            "slab_warp_aggregated_kernel_ms": round(_kernel_only_ms(
                lambda: raymarch_backward(go, vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, True, False, gvol=gvol,
                                          quad=quad, gvol_mode=4), reps), 3),
        }
    # ---- texture-filtered forward variant (8-bit hardware weights)
    from nanodrr_gb300.raymarch import TextureVolume

    with torch.no_grad():
        tex = TextureVolume(vol)
        soft, _ = raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd)
        hard, _ = raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, texture=tex)
        texture_variant = {
            "fwd_ms": round(_event_ms(lambda: raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, texture=tex),
                                      max(3, args.steps)), 3),
            "rel_maxabs_vs_software": round(_rel_maxabs(hard, soft), 6),
        }
        tex.close()
        tma, _ = raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, fwd_mode=1)
        plain16, _ = raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, tile=(16, 8, 1))
        tma_variant = {
            "fwd_ms": round(_event_ms(lambda: raymarch_forward(vol, vol, M, srcb, tgtb, stepsz, S, 1, Hd, fwd_mode=1),
                                      max(3, args.steps)), 3),
            "bitwise_equal_to_software": bool(torch.equal(tma, plain16)),
        }
        del soft, hard, tma, plain16
    ref_kernel = None
    if rank == 0 and not args.no_reference_kernel:
        torch.cuda.empty_cache()
        try:
            ref_kernel = reference_triton(args, dev, sub, k_inv, sdd, rt, target, args.steps)
        except Exception as e:  # the reference's kernel failing must not lose this run's line
            ref_kernel = {"unavailable": f"the reference's Triton path raised {type(e).__name__}: {e}"[:300]}
    cpu = parity = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, sub, k_inv, sdd, rt)
        try:
            parity = parity_vs_oracle(args, sub, k_inv, sdd, rt, skips)
        except Exception as e:
            parity = {"error": f"{type(e).__name__}: {e}"[:300]}
    uneven = labels = leval = sparse = single = None
    if not args.no_batched:
        del reg, skips
        torch.cuda.empty_cache()
        uneven = batched_uneven(args, dev)
    if not args.no_extras:
        torch.cuda.empty_cache()
        labels = per_label_forward(dev)
        torch.cuda.empty_cache()
        leval = learned_eval(dev)
        torch.cuda.empty_cache()
        sparse = sparse_phantom_skip(dev)
        torch.cuda.empty_cache()
        single = single_frame_forward(dev, with_reference=not args.no_reference_kernel)
    out = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": round(t_dev / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": BASELINE_HEADLINE,
        "dtype": "f32",
        "data": "synthetic seeded CT phantom (no dataset)",
        "config": {
            "workload": (
                f"registration step: {args.volume} f32 phantom ({args.spacing} mm), {B} poses x "
                f"{Hd}x{Hd} detector ({args.pixel} mm), {S} samples/ray, fwd + NCC + bwd to se(3) "
                "6-vector and volume, " + ("eager steps" if args.no_graph else
                                          "the whole step replayed from a CUDA graph")
            ),
            "method": f"{headline} ({'learned proposal + occupancy check' if headline == 'learned' else headline})",
            "l2": "inputs larger than L2 (volume and its gradient 512 MiB each)",
            "parallelism": f"replicas x{world}",
        },
        "methods_frames_per_s": table,
        "methods_frames_per_s_eager": eager,
        "texture_variant": texture_variant,
        "tma_staged_variant": tma_variant,
        "learned_vs_plain": round(table["learned"] / table["plain"], 3),
        "learned_vs_plain_pose_only": round(table["learned_pose_only"] / table["plain_pose_only"], 3),
        "proposal": {
            "train_poses": args.train_poses,
            "train_rays": args.train_poses * Hd * Hd,
            "epochs": args.prop_epochs,
            "loss_first_last": [round(hist[0], 5), round(hist[-1], 5)],
            "prep_s": round(prep_s, 2),
            "fallback_fraction": round(st[1] / max(1, st[0]), 4),
            "marched_over_box_samples": round(st[2] / max(1, st[3]), 4),
            "occupancy_marched_over_box_samples": round(ost[2] / max(1, ost[3]), 4),
        },
        "samples_per_s": round(n_samp * args.steps * world / t_dev, 1),
        "roofline": roofline,
        "adjoint_warp_aggregation": warp_agg,
        "e2e": e2e,
        # per step: pose, [proposal network and window check (learned)],
        # forward march, NCC moments, statistics, score and adjoint, slab
        # plan, scan and fill, adjoint march, per-pose reduction,
        # quad-gradient fold, pose adjoint
        "gpu_launches": (15 if headline == "learned" else 13) * args.steps,
        "clocks": clk,
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if parity is not None:
        out["parity"] = parity
    if ref_kernel is not None:
        out["reference_triton"] = ref_kernel
        if "frames_per_s" in ref_kernel:
            out["vs_reference_triton"] = round(value / ref_kernel["frames_per_s"], 2)
    if uneven is not None:
        out["batched_uneven"] = uneven
    if labels is not None:
        out["per_label_forward"] = labels
    if leval is not None:
        out["learned_eval_1024"] = leval
    if sparse is not None:
        out["sparse_phantom_skip"] = sparse
    if single is not None:
        out["single_frame_forward"] = single
    if rank == 0:
        print(json.dumps(out), flush=True)


def batched_uneven(args, dev, steps=5):
    """64 requests over three phantom volumes (256^3 @ 1.5 mm, 512x512x300 @
    0.8 mm, 384x384x600 @ 0.7 mm), detectors from {128, 200, 256, 384, 512}^2,
    300-1000 samples/ray, poses as above; forward + pose adjoint. Compares a
    loop of single render calls with the persistent batched launch replayed
    from a CUDA graph (tile shapes from the autotuner)."""
    import numpy as np

    import nanodrr_gb300 as nd
    from nanodrr_gb300 import phantom
    from nanodrr_gb300.autotune import Autotuner
    from nanodrr_gb300.batched import BatchedRenderer, RenderRequest

    specs = [((256, 256, 256), (1.5, 1.5, 1.5)), ((300, 512, 512), (0.8, 0.8, 0.8)), ((600, 384, 384), (0.7, 0.7, 0.7))]
    subs = [phantom.make_phantom(sh, sp, seed=10 + i, device=dev).subject(device=dev) for i, (sh, sp) in enumerate(specs)]
    rng = np.random.default_rng(2024)
    reqs = []
    for i in range(64):
        det = int(rng.choice([128, 200, 256, 384, 512]))
        k_inv, sdd = phantom.detector(sdd=1020.0, pixel=1.2 * 256 / det, height=det, width=det)
        reqs.append(RenderRequest(subs[int(rng.integers(0, 3))], k_inv.to(dev), sdd.to(dev), det, det,
                                  int(rng.integers(300, 1001))))
    poses = phantom.random_poses(64, seed=33).to(dev)
    rays = sum(r.height * r.width for r in reqs)

    # (a) a loop of single render calls: forward + pose backward
    def loop():
        for i, r in enumerate(reqs):
            rt = poses[i : i + 1].clone().requires_grad_(True)
            img = nd.render(r.subject, r.k_inv, rt, r.sdd, r.height, r.width, n_samples=r.n_samples)
            img.sum().backward()

    # (b) persistent batched kernel, whole step in a CUDA graph
    tuner = Autotuner(None, reps=3)
    t0 = time.perf_counter()
    br = BatchedRenderer(reqs, autotuner=tuner)
    tune_s = time.perf_counter() - t0
    pose_in = poses.clone()

    def step():
        br.set_poses(pose_in)
        br.forward()
        br.go_flat.fill_(1.0)
        br.backward()

    step()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / steps

    t_loop = timed(loop)
    t_graph = timed(g.replay)
    shapes = {}
    for sh in br.shapes:
        shapes[str(sh)] = shapes.get(str(sh), 0) + 1
    return {
        "workload": "64 requests, 3 volumes, detectors 128-512^2, 300-1000 samples, fwd + pose bwd",
        "rays_per_step": rays,
        "loop_of_render_calls_frames_per_s": round(64 / t_loop, 1),
        "persistent_graph_frames_per_s": round(64 / t_graph, 1),
        "speedup": round(t_loop / t_graph, 2),
        "autotune_s": round(tune_s, 2),
        "tile_shapes": shapes,
    }


def _event_ms(fn, steps):
    """Median CUDA-event time of `fn` on the current stream (ms), after 3 warm-up calls."""
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def _kernel_only_ms(fn, reps):
    """Median duration (ms) of the ray-march kernel inside `fn`: the library
    records a pair of CUDA events on the launch stream just before and after
    its march kernel (ndrr_set_kernel_events), so the call's other launches
    (gradient zeroing, slab planning, pose reduction, fold) are excluded."""
    import ctypes

    from nanodrr_gb300 import _ffi

    lib = _ffi.load()
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        e1.record()  # creates both events before the library records them
        torch.cuda.synchronize()
        _ffi.check(lib.ndrr_set_kernel_events(ctypes.c_void_p(e0.cuda_event), ctypes.c_void_p(e1.cuda_event)),
                   "ndrr_set_kernel_events")
        try:
            fn()
        finally:
            lib.ndrr_set_kernel_events(None, None)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def l2_read_peak(dev, sizes_mib=(16, 32, 48), passes=256, reps=10, warm_ms=100.0):
    """Measured L2 read bandwidth (GB/s): the library's probe streams an
    L2-resident buffer `passes` times with L2-only loads, CUDA events around
    each launch; the best over `reps` launches of buffers of each size, each
    allocated afresh, after about `warm_ms` of back-to-back launches so the
    clocks have left any idle state (a 2 ms probe read 12 to 20 TB/s on
    different runs)."""
    import ctypes

    from nanodrr_gb300 import _ffi

    lib = _ffi.load()
    sink = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    best = 0.0
    for mib in sizes_mib:
        buf = torch.zeros(mib << 20, dtype=torch.uint8, device=dev)

        def launch():
            _ffi.check(lib.ndrr_l2_read_probe(ctypes.c_void_p(buf.data_ptr()), ctypes.c_uint64(buf.numel()), passes,
                                              ctypes.c_void_p(sink.data_ptr()), ctypes.c_void_p(stream)),
                       "ndrr_l2_read_probe")

        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        launch()
        e1.record()
        torch.cuda.synchronize()
        n_warm = max(3, min(2000, int(warm_ms / max(e0.elapsed_time(e1), 1e-3))))
        for _ in range(n_warm):
            launch()
        torch.cuda.synchronize()
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            launch()
            e1.record()
            torch.cuda.synchronize()
            best = max(best, buf.numel() * passes / (e0.elapsed_time(e1) / 1e3) / 1e9)
        del buf
    sizes = "/".join(str(m) for m in sizes_mib)
    return {"gbs": round(best, 1), "how": f"{sizes} MiB buffers each read {passes}x with ld.global.cg by 4 CTAs x 512 "
            f"threads per SM, best of {reps} per size after ~{warm_ms:.0f} ms of warm-up launches, CUDA events"}


def reduction_peak(dev, mib=64, iters=512, reps=10, warm_ms=100.0):
    """Measured rate (G samples/s) of the volume-gradient scatter's pattern
    alone: the library's probe has every warp scatter an 8 x 4 patch of
    neighbouring cells as two 16-byte reductions per sample into an
    L2-resident quad array; best of `reps` launches after ~`warm_ms` of
    warm-up, CUDA events."""
    import ctypes

    from nanodrr_gb300 import _ffi

    lib = _ffi.load()
    buf = torch.zeros(mib << 20, dtype=torch.uint8, device=dev)
    threads = ctypes.c_int32(0)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def launch():
        _ffi.check(lib.ndrr_reduce_probe(ctypes.c_void_p(buf.data_ptr()), ctypes.c_uint64(buf.numel()), iters,
                                         ctypes.byref(threads), ctypes.c_void_p(stream)), "ndrr_reduce_probe")

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    launch()
    e1.record()
    torch.cuda.synchronize()
    for _ in range(max(3, min(1000, int(warm_ms / max(e0.elapsed_time(e1), 1e-3))))):
        launch()
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        launch()
        e1.record()
        torch.cuda.synchronize()
        best = max(best, threads.value * iters / (e0.elapsed_time(e1) / 1e3) / 1e9)
    del buf
    return {"gsamples_per_s": round(best, 1),
            "how": f"{mib} MiB quad array, {threads.value} threads x {iters} samples, two red.global.add.v4.f32 per "
                   f"sample, warps as 8 x 4 patches of cells, best of {reps} after ~{warm_ms:.0f} ms of warm-up"}


def _rays(sub, rt, k_inv, sdd, det, S):
    from nanodrr_gb300.renderer import _affine_product, _make_src, _make_tgt

    dev = rt.device
    M = _affine_product(sub.world_to_voxel[:3], rt).contiguous()
    tgt = _make_tgt(k_inv, sdd, det, det, dev, torch.float32).expand(rt.shape[0], -1, -1).contiguous()
    src = _make_src(False, tgt, sdd).contiguous()
    step = ((tgt - src).norm(dim=-1) / (S - 1)).contiguous()
    return M, src, tgt, step


def _rel_maxabs(a, b):
    """max over images of max|a - b| / max|b| (images = leading dims but the last)."""
    a, b = a.double().flatten(0, -2), b.double().flatten(0, -2)
    b = b.to(a.device)
    num = (a - b).abs().amax(-1)
    den = b.abs().amax(-1).clamp_min(1e-30)
    return float((num / den).max())


def per_label_forward(dev, steps=5):
    """Per-label forward on the 512 x 512 x 400 phantom (0.8 x 0.8 x 1.0 mm),
    8 label channels plus the total, 32 poses, 256^2 detector at 1.2 mm, 800
    samples/ray; the volume as float32 (quad layout, uint8 label gathers) and
    as bf16 (the labelled quad layout that render() uses for it: classes in
    the corner loads), the bf16 volume also with label gathers, and the
    one-channel forward of the same rays for scale."""
    from nanodrr_gb300 import phantom
    from nanodrr_gb300.raymarch import quad_volume, quad_volume_labeled, raymarch_forward
    from nanodrr_gb300.renderer import compact_label

    B, det, S, C = 32, 256, 800, 8
    ph = phantom.make_phantom((400, 512, 512), (0.8, 0.8, 1.0), seed=0, device=dev)
    sub = ph.subject(device=dev, with_labels=True)
    del ph
    lab = compact_label(sub)
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=1.2, height=det, width=det)
    M, src, tgt, step = _rays(sub, phantom.random_poses(B, seed=1).to(dev), k_inv.to(dev), sdd.to(dev), det, S)
    vols = {"f32": sub.image[0, 0].contiguous()}
    vols["bf16"] = vols["f32"].to(torch.bfloat16)
    res = {"workload": "512x512x400 phantom, 8 labels + total, 32 poses, 256^2, 800 samples, forward",
           "l2": "inputs larger than L2"}
    outs = {}
    cases = (("f32", vols["f32"], False), ("bf16", vols["bf16"], True), ("bf16_label_gathers", vols["bf16"], False))
    for name, v, labelled in cases:
        q = quad_volume_labeled(v, lab, C) if labelled else quad_volume(v)
        fn = lambda: raymarch_forward(v, lab, M, src, tgt, step, S, C, det, with_total=True, quad=q)  # noqa: E731
        ms = _event_ms(fn, steps)
        outs[name] = fn()
        res[name] = {"ms": round(ms, 3), "frames_per_s": round(B / ms * 1e3, 1)}
        del q
    q = quad_volume(vols["f32"])
    one = lambda: raymarch_forward(vols["f32"], vols["f32"], M, src, tgt, step, S, 1, det, quad=q)  # noqa: E731
    res["one_channel_f32_ms"] = round(_event_ms(one, steps), 3)
    res["bf16_vs_f32_rel_maxabs"] = {
        "channels": round(_rel_maxabs(outs["bf16"][0], outs["f32"][0]), 5),
        "total": round(_rel_maxabs(outs["bf16"][1], outs["f32"][1]), 5),
    }
    res["labelled_quad_equals_label_gathers"] = bool(torch.equal(outs["bf16"][0], outs["bf16_label_gathers"][0]))
    return res


def _skip_kwargs(es, vol, M, src, tgt, step, S, det):
    """Skip arguments of one step's forward and adjoint: the learned
    proposal's windows are computed once and shared by both passes (as
    render() does); the occupancy skip runs inside the march kernels."""
    from nanodrr_gb300 import _ffi
    from nanodrr_gb300.raymarch import skip_windows

    if es is not None and es.mode == _ffi.NDRR_SKIP_PROPOSAL:
        return {"windows": skip_windows(vol, M, src, tgt, step, S, det, es)}
    return {"skip": es}


def single_frame_forward(dev, runs=10, iters=100, warmup=25, with_reference=True):
    """The shape of the reference's published benchmark (tests/benchmark/
    benchmark.py:23-47, 58-96): one AP pose 850 mm from the isocenter, 200^2
    detector at 2.0 mm, sdd 1020, 500 samples, fp32 forward, on the 512 x 512
    x 400 phantom (its CT volume is not available); frames/s timed its way,
    CUDA events around 100 back-to-back render calls, median of 10 runs, so
    host time per call counts. Also the same call replayed from a CUDA graph."""
    import nanodrr_gb300 as nd
    from nanodrr_gb300 import geometry, phantom

    ph = phantom.make_phantom((400, 512, 512), (0.8, 0.8, 1.0), seed=0, device=dev)
    sub = ph.subject(device=dev)
    del ph
    k_inv = geometry.make_k_inv(1020.0, 2.0, 2.0, 0.0, 0.0, 200, 200).to(dev)
    rt = geometry.make_rt_inv(torch.tensor([[0.0, 0.0, 0.0]]), torch.tensor([[0.0, 850.0, 0.0]]), "AP",
                              isocenter=sub.isocenter.cpu()).to(dev)
    sdd = torch.tensor([1020.0], device=dev)

    def wall_us(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(runs):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(iters):
                fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / iters * 1e3)
        return statistics.median(ts)

    with torch.no_grad():
        call = lambda: nd.render(sub, k_inv, rt, sdd, 200, 200, n_samples=500)  # noqa: E731
        eager = wall_us(call)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                call()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            call()
        graphed = wall_us(graph.replay)
        res = {"workload": "1 AP pose, 200^2 detector at 2.0 mm, 500 samples, fp32 forward, 512x512x400 phantom",
               "render_call_us": round(eager, 1), "render_call_frames_per_s": round(1e6 / eager, 1),
               "graph_replay_us": round(graphed, 1), "graph_replay_frames_per_s": round(1e6 / graphed, 1)}
        # the reference's own Triton kernel, the same call timed the same way
        ref, why = load_reference() if with_reference else (None, "not requested")
        if ref is None:
            res["reference_triton"] = {"unavailable": why}
        else:
            rsub = reference_subject(ref, sub._image_hu, sub.world_to_voxel, sub.voxel_to_world, sub.isocenter)
            rcall = lambda: ref["render"](rsub, k_inv, rt, sdd, 200, 200, n_samples=500, backend="triton")  # noqa: E731
            r_us = wall_us(rcall)
            res["reference_triton"] = {"render_call_us": round(r_us, 1), "render_call_frames_per_s": round(1e6 / r_us, 1),
                                       "image_rel_maxabs_vs_this_library": round(_rel_maxabs(call(), rcall()), 8)}
    return res


# ------------------------------------------------ the reference's own kernel
REF_DIR = ROOT / "baseline" / "_ref"


def load_reference():
    """The unmodified reference package from baseline/_ref (installed by
    baseline/install_reference.py) and its Triton backend, or a reason why it
    cannot run here. Triton's bundled ptxas predates sm_103a, so the CUDA
    toolkit's ptxas is named for it (TRITON_PTXAS_PATH) unless one is set."""
    if not (REF_DIR / "nanodrr").is_dir():
        return None, "baseline/_ref is not installed (python baseline/install_reference.py <nanodrr checkout>)"
    if "TRITON_PTXAS_PATH" not in os.environ:
        for cand in (shutil.which("ptxas"), "/usr/local/cuda/bin/ptxas"):
            if cand and Path(cand).exists():
                os.environ["TRITON_PTXAS_PATH"] = cand
                break
    try:
        import triton  # noqa: F401
    except Exception as e:  # pragma: no cover - depends on the host
        return None, f"triton is not importable: {e}"
    if str(REF_DIR) not in sys.path:
        sys.path.insert(0, str(REF_DIR))
    try:
        from nanodrr.data import Subject as RefSubject
        from nanodrr.drr.renderer import _triton_available
        from nanodrr.drr.renderer import render as ref_render
        from nanodrr.metrics import NormalizedCrossCorrelation2d as RefNCC
    except Exception as e:
        return None, f"the reference does not import: {e}"
    if not _triton_available():
        return None, "the reference's Triton backend does not import"
    return {"Subject": RefSubject, "render": ref_render, "NCC": RefNCC}, None


def reference_subject(ref, image, world_to_voxel, voxel_to_world, isocenter):
    """The reference's Subject around a [1, 1, D, H, W] attenuation volume."""
    return ref["Subject"](
        imagedata=image,
        labeldata=torch.zeros_like(image.detach()),
        voxel_to_world=voxel_to_world,
        world_to_voxel=world_to_voxel,
        voxel_to_grid=ref["Subject"]._make_voxel_to_grid(image.shape).to(image.device),
        isocenter=isocenter,
        max_label=0,
        convert_to_mu=False,
    )


def reference_triton(args, dev, sub, k_inv, sdd, rt, target, steps):
    """The reference's fused Triton kernel on this GPU through its own
    render(..., backend="triton") and NormalizedCrossCorrelation2d, on the
    headline workload: fwd + NCC + bwd to the pose (its rt_inv; the se(3)
    chain of its Registration module needs roma, which is not installed) and
    to the volume, CUDA events around `steps` eager steps after the same
    warm-up; plus the forward alone and parity of its image and gradients
    with this library's on the same inputs."""
    import nanodrr_gb300 as nd
    from nanodrr_gb300.registration import NormalizedCrossCorrelation2d

    ref, why = load_reference()
    if ref is None:
        return {"unavailable": why}
    B, Hd, S = rt.shape[0], args.det, args.samples
    vol_leaf = sub._image_hu.detach().clone().requires_grad_(True)
    rsub = reference_subject(ref, vol_leaf, sub.world_to_voxel, sub.voxel_to_world, sub.isocenter)
    rncc = ref["NCC"]()
    rt_leaf = rt.detach().clone().requires_grad_(True)

    def step():
        vol_leaf.grad = None
        rt_leaf.grad = None
        img = ref["render"](rsub, k_inv, rt_leaf, sdd, Hd, Hd, n_samples=S, backend="triton")
        loss = -rncc(img, target).mean()
        loss.backward()
        return loss

    t0 = time.perf_counter()
    step()
    torch.cuda.synchronize()
    compile_s = time.perf_counter() - t0
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    step_s = e0.elapsed_time(e1) / 1e3 / steps
    with torch.no_grad():
        fwd = lambda: ref["render"](rsub, k_inv, rt, sdd, Hd, Hd, n_samples=S, backend="triton")  # noqa: E731
        fwd_ms = _event_ms(fwd, max(3, steps))
        ref_img = fwd()
    # the same step through this library (render + NCC kernels) for parity
    step()
    g_rt_ref, g_vol_ref = rt_leaf.grad.clone(), vol_leaf.grad.clone()
    keep = sub._image_hu
    mine_vol = sub._image_hu.detach().clone().requires_grad_(True)
    sub._image_hu = mine_vol
    try:
        rt_mine = rt.detach().clone().requires_grad_(True)
        img = nd.render(sub, k_inv, rt_mine, sdd, Hd, Hd, n_samples=S)
        (-NormalizedCrossCorrelation2d()(img, target).mean()).backward()
    finally:
        sub._image_hu = keep
    res = {
        "impl": "reference render(..., backend='triton') from baseline/_ref, unmodified; TRITON_PTXAS_PATH = "
                + os.environ.get("TRITON_PTXAS_PATH", "default"),
        "frames_per_s": round(B / step_s, 2),
        "ms_per_step": round(step_s * 1e3, 3),
        "fwd_frames_per_s": round(B / fwd_ms * 1e3, 2),
        "first_call_s": round(compile_s, 2),
        "parity_vs_this_library": {
            "image_rel_maxabs": round(_rel_maxabs(img.detach(), ref_img), 8),
            "pose_grad_rel_maxabs": round(_rel_maxabs(rt_mine.grad[:, :3].reshape(1, -1),
                                                      g_rt_ref[:, :3].reshape(1, -1)), 8),
            "volume_grad_rel_maxabs": round(_rel_maxabs(mine_vol.grad.reshape(1, -1),
                                                        g_vol_ref.reshape(1, -1)), 8),
        },
    }
    del rsub, vol_leaf, mine_vol
    return res


def sparse_phantom_skip(dev, steps=5, epochs=40, body_scale=0.4, train_poses=64):
    """Plain vs occupancy vs learned skipping on a sparser phantom: the same
    512^3 recipe with the body scaled to 0.4 of the extent (more air along
    every ray), 32 poses x 256^2 x 800 samples, forward + backward; the
    network is trained on 64 other poses (a small body needs more poses than
    the full-size one to place its silhouette: 27 % of rays fell back with 16,
    10 % with 64). Not the headline workload: it shows what exact skipping
    gains when there is air to skip."""
    from nanodrr_gb300 import phantom
    from nanodrr_gb300.empty_space import EmptySpace, train_proposal
    from nanodrr_gb300.raymarch import quad_volume, raymarch_backward, raymarch_forward

    ph = phantom.make_phantom((512, 512, 512), (0.8, 0.8, 1.0), seed=0, device=dev, body_scale=body_scale)
    sub = ph.subject(device=dev)
    del ph
    vol = sub.image[0, 0].contiguous()
    q = quad_volume(vol)
    B, det, S = 32, 256, 800
    k_inv, sdd = phantom.detector(sdd=1020.0, pixel=1.2, height=det, width=det)
    k_inv, sdd = k_inv.to(dev), sdd.to(dev)
    Mt, srct, tgtt, stept = _rays(sub, phantom.random_poses(train_poses, seed=500).to(dev), k_inv, sdd, det, S)
    net, _ = train_proposal(vol, Mt, srct, tgtt, stept, S, det, epochs=epochs, batch=65536, lr=2e-3, alpha=20.0)
    del Mt, srct, tgtt, stept
    M, src, tgt, step = _rays(sub, phantom.random_poses(B, seed=1).to(dev), k_inv, sdd, det, S)
    go = torch.randn(B, 1, det * det, device=dev)
    gvol = torch.zeros_like(vol)
    skips = {"plain": None, "occupancy": EmptySpace.occupancy(vol, cell=4),
             "learned": EmptySpace.proposal(vol, net, cell=4, margin=2.0)}
    res = {"workload": f"512^3 phantom with the body at {body_scale} of the extent, 32 poses, 256^2, 800 samples, "
                       f"fwd + bwd; network trained on {train_poses} other poses"}
    for name, es in skips.items():
        def pose_step(es=es):
            kw = _skip_kwargs(es, vol, M, src, tgt, step, S, det)
            raymarch_forward(vol, vol, M, src, tgt, step, S, 1, det, quad=q, **kw)
            raymarch_backward(go, vol, vol, M, src, tgt, step, S, 1, det, False, False, quad=q, **kw)

        def full_step(es=es):
            kw = _skip_kwargs(es, vol, M, src, tgt, step, S, det)
            raymarch_forward(vol, vol, M, src, tgt, step, S, 1, det, quad=q, **kw)
            raymarch_backward(go, vol, vol, M, src, tgt, step, S, 1, det, True, False, gvol=gvol, quad=q, **kw)

        entry = {"pose_only_frames_per_s": round(B / _event_ms(pose_step, steps) * 1e3, 1),
                 "with_volume_grad_frames_per_s": round(B / _event_ms(full_step, steps) * 1e3, 1)}
        if es is not None:
            stats = torch.zeros(4, dtype=torch.int64, device=dev)
            raymarch_forward(vol, vol, M, src, tgt, step, S, 1, det, quad=q, skip=es, stats=stats)
            st = stats.tolist()
            entry["fallback_fraction"] = round(st[1] / max(1, st[0]), 4)
            entry["marched_over_box_samples"] = round(st[2] / max(1, st[3]), 4)
        res[name] = entry
    for name in ("occupancy", "learned"):
        res[f"{name}_vs_plain_pose_only"] = round(res[name]["pose_only_frames_per_s"]
                                                  / res["plain"]["pose_only_frames_per_s"], 3)
    return res


def learned_eval(dev, steps=5, epochs=40):
    """Learned proposal against plain and occupancy-only marching: network
    trained on 16 poses x 256^2 rays (about 1e6) of the 512 x 512 x 400
    phantom, evaluated on 8 other poses at a 1024^2 detector with 1000
    samples/ray, forward + backward (pose only, and pose + volume)."""
    from nanodrr_gb300 import phantom
    from nanodrr_gb300.empty_space import EmptySpace, train_proposal
    from nanodrr_gb300.raymarch import quad_volume, raymarch_backward, raymarch_forward

    ph = phantom.make_phantom((400, 512, 512), (0.8, 0.8, 1.0), seed=0, device=dev)
    sub = ph.subject(device=dev)
    del ph
    vol = sub.image[0, 0].contiguous()
    q = quad_volume(vol)
    S_tr, S = 800, 1000
    k_tr, sdd = phantom.detector(sdd=1020.0, pixel=1.2, height=256, width=256)
    Mt, srct, tgtt, stept = _rays(sub, phantom.random_poses(16, seed=500).to(dev), k_tr.to(dev), sdd.to(dev), 256,
                                  S_tr)
    t0 = time.perf_counter()
    net, hist = train_proposal(vol, Mt, srct, tgtt, stept, S_tr, 256, epochs=epochs, batch=65536, lr=2e-3,
                               alpha=20.0)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del Mt, srct, tgtt, stept
    B, det = 8, 1024
    k_ev, sdd = phantom.detector(sdd=1020.0, pixel=1.2 * 256 / det, height=det, width=det)
    M, src, tgt, step = _rays(sub, phantom.random_poses(B, seed=7).to(dev), k_ev.to(dev), sdd.to(dev), det, S)
    go = torch.randn(B, 1, det * det, device=dev)
    gvol = torch.zeros_like(vol)
    skips = {"plain": None, "occupancy": EmptySpace.occupancy(vol, cell=4),
             "learned": EmptySpace.proposal(vol, net, cell=4, margin=2.0)}
    res = {"workload": "512x512x400 phantom, 8 poses, 1024^2 detector, 1000 samples, fwd + bwd",
           "train_rays": 16 * 256 * 256, "train_s": round(train_s, 2)}
    ref = None
    for name, es in skips.items():
        def pose_step(es=es):
            kw = _skip_kwargs(es, vol, M, src, tgt, step, S, det)
            raymarch_forward(vol, vol, M, src, tgt, step, S, 1, det, quad=q, **kw)
            return raymarch_backward(go, vol, vol, M, src, tgt, step, S, 1, det, False, False, quad=q, **kw)

        def full_step(es=es):
            kw = _skip_kwargs(es, vol, M, src, tgt, step, S, det)
            raymarch_forward(vol, vol, M, src, tgt, step, S, 1, det, quad=q, **kw)
            return raymarch_backward(go, vol, vol, M, src, tgt, step, S, 1, det, True, False, gvol=gvol, quad=q,
                                     **kw)

        ms_pose = _event_ms(pose_step, steps)
        ms_full = _event_ms(full_step, steps)
        stats = torch.zeros(4, dtype=torch.int64, device=dev)
        out, _ = raymarch_forward(vol, vol, M, src, tgt, step, S, 1, det, quad=q, skip=es, stats=stats)
        gM = pose_step()[1]
        entry = {"pose_only_frames_per_s": round(B / ms_pose * 1e3, 1),
                 "with_volume_grad_frames_per_s": round(B / ms_full * 1e3, 1)}
        if es is not None:
            st = stats.tolist()
            entry["fallback_fraction"] = round(st[1] / max(1, st[0]), 4)
            entry["marched_over_box_samples"] = round(st[2] / max(1, st[3]), 4)
        if ref is None:
            ref = (out, gM)
        else:
            entry["rel_maxabs_vs_plain"] = {"image": _rel_maxabs(out, ref[0]),
                                            "pose_grad": _rel_maxabs(gM.flatten(1), ref[1].flatten(1))}
        res[name] = entry
    res["learned_vs_plain_pose_only"] = round(res["learned"]["pose_only_frames_per_s"]
                                              / res["plain"]["pose_only_frames_per_s"], 3)
    res["learned_vs_occupancy_pose_only"] = round(res["learned"]["pose_only_frames_per_s"]
                                                  / res["occupancy"]["pose_only_frames_per_s"], 3)
    return res


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "source": "fallback"}


# ----------------------------------------------------------- CPU baseline
def _cpu_sample(args, vol_cpu, w2v, k_inv, sdd, rt, rays):
    """One bounded sample: `rays` rays of pose 0, forward + backward to the pose
    and the volume through the restated reference CPU path (fp32)."""
    from oracle import make_src, make_tgt, render_oracle

    Hd = args.det
    tgt_full = make_tgt(k_inv.cpu(), sdd.cpu(), Hd, Hd, torch.float32)
    g = torch.Generator().manual_seed(0)
    idx = torch.randperm(Hd * Hd, generator=g)[:rays]
    tgt = tgt_full[:, idx]
    src = make_src(False, tgt, sdd.cpu())
    rtp = rt[:1].cpu().clone().requires_grad_(True)
    vol = vol_cpu
    vol.grad = None
    out = render_oracle(vol, None, w2v, rtp, src, tgt, args.samples, 1)
    out.sum().backward()
    return out


def parity_vs_oracle(args, sub, k_inv, sdd, rt, skips, poses=2, rays=2048):
    """FP64 parity of the headline workload, computed in the CPU-baseline leg
    where the oracle is the checker: a seeded subset of `rays` pixels of each
    of the first `poses` poses is rendered by the CUDA path (plain march and
    learned proposal) with gradients to rt_inv and to the volume of a
    positively weighted ray sum, and by the float64 restatement of the
    reference's PyTorch backend on the host from the same float32 inputs;
    relative max-abs errors (image per pose, gradients overall)."""
    import nanodrr_gb300 as nd
    from nanodrr_gb300.renderer import _make_tgt
    from oracle import render_oracle

    dev = rt.device
    Hd, S = args.det, args.samples
    g = torch.Generator().manual_seed(11)
    idx = torch.stack([torch.randperm(Hd * Hd, generator=g)[:rays] for _ in range(poses)])
    tgt = _make_tgt(k_inv, sdd, Hd, Hd, dev, torch.float32)[0][idx.to(dev)].contiguous()
    src = torch.zeros(poses, 1, 3, device=dev)
    tgt64 = _make_tgt(k_inv.double().cpu(), sdd.double().cpu(), Hd, Hd, "cpu", torch.float64)[0][idx]
    src64 = torch.zeros(poses, 1, 3, dtype=torch.float64)
    weight = 0.5 + torch.rand(poses, 1, rays, generator=g, dtype=torch.float64)
    vol64 = sub._image_hu.detach()[0, 0].double().cpu().requires_grad_(True)
    w2v64 = sub.world_to_voxel.double().cpu()
    rt64 = rt[:poses].detach().double().cpu().requires_grad_(True)
    ref = render_oracle(vol64, None, w2v64, rt64, src64, tgt64, S)
    (ref * weight).sum().backward()
    ref = ref.detach()
    res = {"oracle": "float64 restatement of the reference's PyTorch backend on the host, same float32 inputs",
           "rays": f"{rays} seeded pixels of each of the first {poses} poses, {S} samples",
           "tolerances": {"image": 1e-5, "gradients": 1e-3}}
    keep = sub._image_hu
    w = weight.float().to(dev)
    for name in ("plain", "learned"):
        vol = keep.detach().clone().requires_grad_(True)
        sub._image_hu = vol
        sub.empty_space = skips[name]
        try:
            rtp = rt[:poses].detach().clone().requires_grad_(True)
            out = nd.render(sub, k_inv, rtp, sdd, rays // 64, 64, n_samples=S, src=src, tgt=tgt)
            out = out.reshape(poses, 1, rays)
            (out * w).sum().backward()
        finally:
            sub._image_hu = keep
            sub.empty_space = None
        res[name] = {
            "image_rel_maxabs": _rel_maxabs(out.detach().double().cpu()[:, 0], ref[:, 0]),
            "pose_grad_rel_maxabs": _rel_maxabs(rtp.grad[:, :3].reshape(1, -1).double().cpu(),
                                                rt64.grad[:, :3].reshape(1, -1)),
            "volume_grad_rel_maxabs": _rel_maxabs(vol.grad.reshape(1, -1).double().cpu(),
                                                  vol64.grad.reshape(1, -1)),
        }
    return res


def cpu_baseline(args, sub, k_inv, sdd, rt):
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    vol_cpu = sub.image[0, 0].detach().float().cpu().requires_grad_(True)
    w2v = sub.world_to_voxel.detach().float().cpu()
    rays = args.cpu_rays
    _cpu_sample(args, vol_cpu, w2v, k_inv, sdd, rt, max(64, rays // 8))  # warm-up
    times = []
    t_end = time.perf_counter() + 15.0
    while len(times) < 3 or (time.perf_counter() < t_end and len(times) < 10):
        t0 = time.perf_counter()
        _cpu_sample(args, vol_cpu, w2v, k_inv, sdd, rt, rays)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    frames_per_s = (rays / (args.det * args.det)) / t
    return {
        "value": round(frames_per_s, 4),
        "unit": "frames/s",
        "cores": threads,
        "kind": "port",
        "sample": (
            f"{rays} of {args.det * args.det} rays of one pose, {args.samples} samples, fp32 forward + backward to "
            f"pose and volume via torch grid_sample on CPU (the reference's PyTorch backend restated), median of "
            f"{len(times)}; frames/s = ray fraction / time"
        ),
    }


def run_reference(args, world, rank, local):
    if rank != 0:
        return
    dev = torch.device("cuda", local) if torch.cuda.is_available() else torch.device("cpu")
    ph, k_inv, sdd, rt, held = workload(args, dev)
    sub = ph.subject(device="cpu")
    del ph
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    vol_cpu = sub.image[0, 0].detach().float().requires_grad_(True)
    w2v = sub.world_to_voxel.float()
    rays = args.cpu_rays
    for _ in range(max(args.warmup, 1)):
        _cpu_sample(args, vol_cpu, w2v, k_inv, sdd, rt, rays)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _cpu_sample(args, vol_cpu, w2v, k_inv, sdd, rt, rays)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    frames = args.steps * rays / (args.det * args.det)
    value = frames / total
    out = {
        "metric": METRIC,
        "impl": "reference",
        "value": round(value, 4),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic seeded CT phantom (no dataset)",
        "config": {
            "workload": (
                f"registration step: {args.volume} f32 phantom ({args.spacing} mm), {args.batch} poses x "
                f"{args.det}x{args.det} detector ({args.pixel} mm), {args.samples} samples/ray, fwd + bwd to pose "
                "and volume"
            ),
            "method": "the reference's PyTorch backend (grid_sample), restated, on the host cores",
            "sample_per_step": f"{rays} rays of one pose, scaled to frames/s",
        },
        "cpu_baseline": {
            "value": round(value, 4),
            "unit": "frames/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{rays} rays x {args.samples} samples per step, torch grid_sample on CPU (reference PyTorch "
            "backend restated)",
        },
        "e2e": {"value": round(value, 4), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
