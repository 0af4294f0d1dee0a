"""Registration step around `render`: pose perturbation and NCC loss.

`Registration` mirrors the reference's module (nanodrr
src/nanodrr/registration/registration.py:9-84): the optimisable so(3)
rotation vector and translation perturb the initial pose about the
volume's isocenter, pose = rt_inv @ pivot @ T(rot, xyz) @ pivot^-1.
`NormalizedCrossCorrelation2d` mirrors src/nanodrr/metrics/ncc.py:8-37
(per-image zero-mean, unit-variance correlation, optional patches).
On CUDA the pose and its adjoint run in the library's kernels
(`ndrr_pose_so3_fwd/bwd`), as do the NCC score and its gradient
(`ndrr_ncc_fwd/bwd`), like the render and its adjoint. `GraphedStep` replays a whole step (pose, render,
loss, backward) from a CUDA graph.
"""

from __future__ import annotations

import ctypes

import torch

from . import _ffi
from .geometry import convert, mm_small, transform_point
from .renderer import build_quad, quad_cache_key, render


class Registration(torch.nn.Module):
    def __init__(self, subject, rt_inv, k_inv, sdd, height, width, eps: float = 1e-8, batch: int | None = None):
        super().__init__()
        self.subject = subject
        self.register_buffer("rt_inv", rt_inv)
        self.register_buffer("k_inv", k_inv)
        self.register_buffer("sdd", sdd)
        self.height = height
        self.width = width
        # isocenter in camera coordinates; the 4x4 inverse is taken on the host
        # in float64 (tiny, and it keeps CUDA linear-algebra libraries out of
        # the render path)
        inv = torch.linalg.inv(rt_inv.detach().double().cpu()).to(rt_inv)
        c = transform_point(inv, subject.isocenter[None].expand(rt_inv.shape[0], 3)[:, None])[:, 0]
        self.register_buffer("pivot", self._make_translation(c))
        self.register_buffer("pivot_inv", self._make_translation(-c))
        nb = batch if batch is not None else 1
        self._rot = torch.nn.Parameter(eps * torch.randn(nb, 3, device=c.device))
        self._xyz = torch.nn.Parameter(eps * torch.randn(nb, 3, device=c.device))

    @property
    def pose(self) -> torch.Tensor:
        """Change of basis about the isocenter: rt_inv @ pivot @ T @ pivot_inv
        (reference registration.py:64-68). On CUDA one kernel evaluates it
        and its adjoint (`ndrr_pose_so3_fwd/bwd`); on the host it is composed
        from torch ops."""
        if self.rt_inv.is_cuda:
            return so3_pose(self._rot, self._xyz, self.rt_inv, self.pivot, self.pivot_inv)
        T = convert(self._rot, self._xyz, "so3_log")
        return mm_small(mm_small(mm_small(self.rt_inv, self.pivot), T), self.pivot_inv)

    def forward(self, n_samples: int = 500, backend: str = "auto") -> torch.Tensor:
        return render(self.subject, self.k_inv, self.pose, self.sdd, self.height, self.width, n_samples,
                      backend=backend)

    @torch.no_grad()
    def rescale_(self, scale: float) -> None:
        """Change the rendering resolution by rescaling the camera's
        intrinsics (reference registration.py:70-76)."""
        self.k_inv[..., 0, 0] /= scale
        self.k_inv[..., 1, 1] /= scale
        self.height = int(round(self.height * scale))
        self.width = int(round(self.width * scale))

    @staticmethod
    def _make_translation(t: torch.Tensor) -> torch.Tensor:
        T = torch.eye(4, device=t.device, dtype=t.dtype)[None].repeat(len(t), 1, 1)
        T[:, :3, 3] = t
        return T


def _pose_inputs(rot, xyz, rt_inv, pivot, pivot_inv):
    B = rt_inv.shape[0]
    rows = rot.shape[0]
    if rot.shape != (rows, 3) or xyz.shape != (rows, 3) or rows not in (1, B):
        raise ValueError(f"rot and xyz must be [1 or B, 3] with B = {B}, got {tuple(rot.shape)}, {tuple(xyz.shape)}")
    for name, m in (("rt_inv", rt_inv), ("pivot", pivot), ("pivot_inv", pivot_inv)):
        if m.shape != (B, 4, 4):
            raise ValueError(f"{name} must be [{B}, 4, 4], got {tuple(m.shape)}")
    f = lambda t: t.detach().float().contiguous()  # noqa: E731
    return B, rows, f(rot), f(xyz), f(rt_inv), f(pivot), f(pivot_inv)


@torch.library.custom_op("nanodrr_gb300::so3_pose", mutates_args=())
def _so3_pose_op(rot: torch.Tensor, xyz: torch.Tensor, rt_inv: torch.Tensor, pivot: torch.Tensor,
                 pivot_inv: torch.Tensor) -> torch.Tensor:
    B, rows, r, x, a, p, c = _pose_inputs(rot, xyz, rt_inv, pivot, pivot_inv)
    pose = torch.empty(B, 4, 4, device=rt_inv.device)
    _ffi.check(_ffi.load().ndrr_pose_so3_fwd(r.data_ptr(), x.data_ptr(), rows, a.data_ptr(), p.data_ptr(),
                                             c.data_ptr(), B, pose.data_ptr(),
                                             torch.cuda.current_stream(rt_inv.device).cuda_stream),
               "ndrr_pose_so3_fwd")
    return pose.to(rt_inv.dtype)


@_so3_pose_op.register_fake
def _(rot, xyz, rt_inv, pivot, pivot_inv):
    return rt_inv.new_empty(rt_inv.shape[0], 4, 4)


@torch.library.custom_op("nanodrr_gb300::so3_pose_bwd", mutates_args=())
def _so3_pose_bwd_op(gpose: torch.Tensor, rot: torch.Tensor, xyz: torch.Tensor, rt_inv: torch.Tensor,
                     pivot: torch.Tensor, pivot_inv: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    B, rows, r, x, a, p, c = _pose_inputs(rot, xyz, rt_inv, pivot, pivot_inv)
    g = gpose.float().contiguous()
    g_rot = torch.empty(B, 3, device=rt_inv.device)
    g_xyz = torch.empty(B, 3, device=rt_inv.device)
    _ffi.check(_ffi.load().ndrr_pose_so3_bwd(g.data_ptr(), r.data_ptr(), x.data_ptr(), rows, a.data_ptr(),
                                             p.data_ptr(), c.data_ptr(), B, g_rot.data_ptr(), g_xyz.data_ptr(),
                                             torch.cuda.current_stream(rt_inv.device).cuda_stream),
               "ndrr_pose_so3_bwd")
    if rows == 1 and B > 1:  # a broadcast parameter: sum over the poses
        g_rot, g_xyz = g_rot.sum(0, keepdim=True), g_xyz.sum(0, keepdim=True)
    return g_rot, g_xyz


@_so3_pose_bwd_op.register_fake
def _(gpose, rot, xyz, rt_inv, pivot, pivot_inv):
    return rot.new_empty(rot.shape, dtype=torch.float32), xyz.new_empty(xyz.shape, dtype=torch.float32)


def _so3_pose_setup(ctx, inputs, output):
    ctx.save_for_backward(*inputs)


def _so3_pose_backward(ctx, gpose):
    rot, xyz, rt_inv, pivot, pivot_inv = ctx.saved_tensors
    if any(ctx.needs_input_grad[2:]):
        raise RuntimeError("so3_pose differentiates the rotation and translation only; rt_inv, pivot and "
                           "pivot_inv are fixed buffers")
    g_rot, g_xyz = _so3_pose_bwd_op(gpose, rot, xyz, rt_inv, pivot, pivot_inv)
    return g_rot.to(rot.dtype), g_xyz.to(xyz.dtype), None, None, None


torch.library.register_autograd("nanodrr_gb300::so3_pose", _so3_pose_backward, setup_context=_so3_pose_setup)


def so3_pose(rot: torch.Tensor, xyz: torch.Tensor, rt_inv: torch.Tensor, pivot: torch.Tensor,
             pivot_inv: torch.Tensor) -> torch.Tensor:
    """rt_inv @ pivot @ T(rot, xyz) @ pivot_inv [B, 4, 4] with T the so3_log
    pose (R = exp([rot]x), t = R xyz), differentiable in rot and xyz
    ([1 or B, 3]); one CUDA kernel each way (`ndrr_pose_so3_fwd/bwd`)."""
    return _so3_pose_op(rot, xyz, rt_inv, pivot, pivot_inv)


class NormalizedCrossCorrelation2d(torch.nn.Module):
    """Score in [-1, 1] per image pair: mean of the product of the two images
    after each is normalised to zero mean and unit variance (+eps), per
    channel, or per p x p window with `patch_size` (the windows are unfolded
    into channels first). Computed by the library's NCC kernels
    (`ndrr_ncc_fwd/bwd`), differentiable in both images."""

    def __init__(self, patch_size: int | None = None, eps: float = 1e-7):
        super().__init__()
        self.patch_size = patch_size
        self.eps = eps

    def forward(self, x1: torch.Tensor, x2: torch.Tensor) -> torch.Tensor:
        if self.patch_size is not None:
            x1, x2 = _to_patches(x1, self.patch_size), _to_patches(x2, self.patch_size)
        if x1.shape != x2.shape:
            raise ValueError("Input images must be the same size")
        return ncc_score(x1, x2, float(self.eps))


def _ncc_check(x1: torch.Tensor, x2: torch.Tensor) -> None:
    if not x1.is_cuda or not x2.is_cuda:
        raise RuntimeError("nanodrr_gb300 computes NCC on CUDA devices only")
    if x1.dim() != 4 or x1.shape != x2.shape:
        raise ValueError(f"NCC takes two [B, C, H, W] images of one shape, got {tuple(x1.shape)}, {tuple(x2.shape)}")


@torch.library.custom_op("nanodrr_gb300::ncc", mutates_args=())
def _ncc_op(x1: torch.Tensor, x2: torch.Tensor, eps: float) -> tuple[torch.Tensor, torch.Tensor]:
    """(score [B], per-plane moments [B, C, 8]) of two [B, C, H, W] images."""
    _ncc_check(x1, x2)
    B, C, H, W = x1.shape
    a, b = x1.float().contiguous(), x2.float().contiguous()
    score = torch.empty(B, device=x1.device)
    stats = torch.empty(B, C, 8, device=x1.device)
    lib = _ffi.load()
    nb = ctypes.c_uint64(0)
    _ffi.check(lib.ndrr_ncc_workspace_bytes(B, C, H * W, ctypes.byref(nb)), "ndrr_ncc_workspace_bytes")
    ws = torch.empty(max(int(nb.value), 16), device=x1.device, dtype=torch.uint8)
    _ffi.check(lib.ndrr_ncc_fwd(a.data_ptr(), b.data_ptr(), B, C, H * W, eps, score.data_ptr(), stats.data_ptr(),
                                ws.data_ptr(), ws.numel(), torch.cuda.current_stream(x1.device).cuda_stream),
               "ndrr_ncc_fwd")
    return score.to(x1.dtype), stats


@_ncc_op.register_fake
def _(x1, x2, eps):
    B, C = x1.shape[:2]
    return x1.new_empty(B), x1.new_empty(B, C, 8, dtype=torch.float32)


@torch.library.custom_op("nanodrr_gb300::ncc_bwd", mutates_args=())
def _ncc_bwd_op(go: torch.Tensor, x1: torch.Tensor, x2: torch.Tensor, stats: torch.Tensor, need1: bool,
                need2: bool) -> tuple[torch.Tensor, torch.Tensor]:
    B, C, H, W = x1.shape
    a, b = x1.float().contiguous(), x2.float().contiguous()
    g1 = torch.empty_like(a) if need1 else a.new_empty(0)
    g2 = torch.empty_like(b) if need2 else b.new_empty(0)
    lib = _ffi.load()
    _ffi.check(lib.ndrr_ncc_bwd(go.float().contiguous().data_ptr(), a.data_ptr(), b.data_ptr(),
                                stats.contiguous().data_ptr(), B, C, H * W, g1.data_ptr() if need1 else None,
                                g2.data_ptr() if need2 else None, torch.cuda.current_stream(x1.device).cuda_stream),
               "ndrr_ncc_bwd")
    return g1, g2


@_ncc_bwd_op.register_fake
def _(go, x1, x2, stats, need1, need2):
    return (torch.empty_like(x1, dtype=torch.float32) if need1 else x1.new_empty(0, dtype=torch.float32),
            torch.empty_like(x2, dtype=torch.float32) if need2 else x2.new_empty(0, dtype=torch.float32))


def _ncc_setup(ctx, inputs, output):
    x1, x2, _ = inputs
    ctx.save_for_backward(x1, x2, output[1])


def _ncc_backward(ctx, g_score, _g_stats):
    x1, x2, stats = ctx.saved_tensors
    need1, need2 = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
    g1, g2 = _ncc_bwd_op(g_score, x1, x2, stats, need1, need2)
    return (g1.to(x1.dtype) if need1 else None, g2.to(x2.dtype) if need2 else None, None)


torch.library.register_autograd("nanodrr_gb300::ncc", _ncc_backward, setup_context=_ncc_setup)


def ncc_score(x1: torch.Tensor, x2: torch.Tensor, eps: float = 1e-7) -> torch.Tensor:
    """NCC score [B] of two [B, C, H, W] image batches (reference
    metrics/ncc.py:18-37 without patches)."""
    return _ncc_op(x1, x2, eps)[0]


def _to_patches(x: torch.Tensor, p: int) -> torch.Tensor:
    """[B, C, H, W] -> [B, C * H' * W', p, p]: every p x p window becomes a
    channel, so the normalisation runs within each window (local NCC), the
    layout the reference produces at ncc.py:65-74."""
    x = x.unfold(2, p, step=1).unfold(3, p, step=1).contiguous()
    b, c, h, w, p1, p2 = x.shape
    return x.reshape(b, c * h * w, p1, p2)


class GraphedStep:
    """One registration step — pose, render, loss and backward — captured in
    a CUDA graph and replayed: the step's ~100 small torch launches and the
    Python autograd pass cost no host time per step, so the GPU runs the
    render kernels back to back.

    `loss_fn(image, target)` returns a scalar. The pose parameters of `reg`
    (and the subject's volume, if it requires a gradient) are the graph's
    static inputs: change them in place (`copy_`) between replays; replacing
    the subject's volume with another tensor makes `replay()` raise
    RuntimeError (the graph would still read the old memory). After each
    `replay()`, `loss` holds the step's loss and `grads` (the parameters'
    `.grad` tensors at capture: pose rotation, translation, then the volume
    when it requires a gradient) its gradients, overwritten by each replay.
    Everything the render call does runs on the current stream without host
    synchronisation or device allocation inside the C library, which is what
    makes it capturable."""

    def __init__(self, reg: Registration, loss_fn, target: torch.Tensor, n_samples: int = 500, warmup: int = 3):
        self.reg = reg
        self.loss_fn = loss_fn
        self.target = target
        self.n_samples = n_samples
        self.params = [p for p in list(reg.parameters()) + [reg.subject._image_hu] if p.requires_grad]
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self._zero()
                self._step()
        torch.cuda.current_stream().wait_stream(side)
        self._zero()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.loss = self._step()
        # the graph's own gradient tensors (a later capture may rebind .grad)
        self.grads = [p.grad for p in self.params]
        # The quad copy of the volume the graph reads: held here (an eager
        # render after a volume change replaces the subject's cached copy),
        # and rebuilt in place before a replay when the volume has changed,
        # like the empty-space grid the graph reads.
        sub = reg.subject
        cache = getattr(sub, "_ndrr_quad_cache", None)
        self._quad = cache[1] if cache is not None else None
        self._quad_labels = (cache[2], cache[3]) if cache is not None else (None, 1)
        # The volume tensor the graph reads, held so that its memory cannot be
        # freed and handed to another tensor while the graph can replay.
        self._vol = sub.image
        self._vol_version = self._vol._version

    def _zero(self):
        for p in self.params:
            p.grad = None

    def _step(self) -> torch.Tensor:
        img = self.reg(n_samples=self.n_samples)
        loss = self.loss_fn(img, self.target)
        loss.backward()
        return loss.detach()

    def _refresh(self):
        sub = self.reg.subject
        img = sub.image
        if img.data_ptr() != self._vol.data_ptr() or img.shape != self._vol.shape or img.dtype != self._vol.dtype:
            raise RuntimeError(
                "the subject's volume is not the tensor this graph was captured with (a new tensor was assigned, "
                "or the HU -> mu conversion produced a new one); build a new GraphedStep, or update the captured "
                "volume in place instead"
            )
        if img._version == self._vol_version:
            return
        vol = img.reshape(img.shape[-3:]) if img.shape[:2] == (1, 1) else img[0, 0]
        if self._quad is not None:
            lab, n_classes = self._quad_labels
            build_quad(vol, lab, n_classes, out=self._quad)
            object.__setattr__(sub, "_ndrr_quad_cache",
                               (quad_cache_key(vol, lab, n_classes), self._quad, lab, n_classes))
        skip = getattr(sub, "empty_space", None)
        if skip is not None:
            skip.grid.refresh(vol)
        self._vol_version = img._version

    def replay(self) -> torch.Tensor:
        self._refresh()
        self.graph.replay()
        return self.loss
