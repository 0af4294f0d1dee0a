"""Registration step around `render`: pose perturbation and NCC loss.

`Registration` mirrors the reference's module (nanodrr
src/nanodrr/registration/registration.py:9-84): the optimisable so(3)
rotation vector and translation perturb the initial pose about the
volume's isocenter, pose = rt_inv @ pivot @ T(rot, xyz) @ pivot^-1.
`NormalizedCrossCorrelation2d` mirrors src/nanodrr/metrics/ncc.py:8-37
(per-image zero-mean, unit-variance correlation, optional patches).
The pose composition is host-side torch (3x3/4x4 products); the NCC score
and its gradient run in the library's kernels (`ndrr_ncc_fwd/bwd`), like the
render and its adjoint. `GraphedStep` replays a whole step (pose, render,
loss, backward) from a CUDA graph.
"""

from __future__ import annotations

import ctypes

import torch

from . import _ffi
from .geometry import convert, mm_small, transform_point
from .renderer import render


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
        T = convert(self._rot, self._xyz, "so3_log")
        return mm_small(mm_small(mm_small(self.rt_inv, self.pivot), T), self.pivot_inv)

    def forward(self, n_samples: int = 500, backend: str = "auto") -> torch.Tensor:
        return render(self.subject, self.k_inv, self.pose, self.sdd, self.height, self.width, n_samples,
                      backend=backend)

    @staticmethod
    def _make_translation(t: torch.Tensor) -> torch.Tensor:
        T = torch.eye(4, device=t.device, dtype=t.dtype)[None].repeat(len(t), 1, 1)
        T[:, :3, 3] = t
        return T


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
    static inputs: change them in place (`copy_`) between replays. After each
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

    def _zero(self):
        for p in self.params:
            p.grad = None

    def _step(self) -> torch.Tensor:
        img = self.reg(n_samples=self.n_samples)
        loss = self.loss_fn(img, self.target)
        loss.backward()
        return loss.detach()

    def replay(self) -> torch.Tensor:
        self.graph.replay()
        return self.loss
