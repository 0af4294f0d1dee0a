"""Persistent batched rendering of heterogeneous requests.

`BatchedRenderer` renders a fixed list of requests — each its own subject
(volumes of one dtype), detector size, sample count and pose — with ONE
persistent kernel launch for the forward and one (+ a small reduction) for the
pose adjoint (`ndrr_batched_fwd/bwd`). Everything the launches read lives in
static device buffers (request descriptors, tile offsets, stacked poses,
outputs, upstream gradients), so a whole step can be captured in a CUDA graph
and replayed with new poses. The reference renders one volume and one
detector size per call (nanodrr src/nanodrr/drr/backends.py:66-69), so a mixed
batch there is a Python loop of launches.

Work order: requests are sorted by cost (rays x samples) so the largest tiles
are taken first and the end of the launch is made of small ones. Tile shapes
come from the autotuner (or a default). With `layout="quad"` (the default)
each subject's quad-layout copy is built once (cached on the subject) and
the requests are marched from it.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _ffi
from .autotune import BATCHED_CANDIDATES, Autotuner
from .raymarch import ndrr_dtype
from .renderer import _affine_product, _camera_rays, cached_quad, compact_label


class Request(ctypes.Structure):
    """Mirror of `ndrr_request`."""

    _fields_ = [
        ("vol", ctypes.c_void_p),
        ("lab", ctypes.c_void_p),
        ("D", ctypes.c_int32),
        ("H", ctypes.c_int32),
        ("W", ctypes.c_int32),
        ("N", ctypes.c_int32),
        ("width", ctypes.c_int32),
        ("n_samples", ctypes.c_int32),
        ("src_per_ray", ctypes.c_int32),
        ("tile_w", ctypes.c_int32),
        ("tile_h", ctypes.c_int32),
        ("sample_split", ctypes.c_int32),
        ("M", ctypes.c_void_p),
        ("src", ctypes.c_void_p),
        ("tgt", ctypes.c_void_p),
        ("step", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
        ("go", ctypes.c_void_p),
        ("gM", ctypes.c_void_p),
        ("gsrc", ctypes.c_void_p),
        ("gtgt", ctypes.c_void_p),
        ("gstep", ctypes.c_void_p),
        ("vol_quad", ctypes.c_void_p),
    ]


class BatchArgs(ctypes.Structure):
    """Mirror of `ndrr_batch_args`."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("abi_version", ctypes.c_uint32),
        ("requests", ctypes.c_void_p),
        ("tile_offsets", ctypes.c_void_p),
        ("n_requests", ctypes.c_int32),
        ("total_tiles", ctypes.c_int32),
        ("vol_dtype", ctypes.c_int32),
        ("lab_dtype", ctypes.c_int32),
        ("go_dtype", ctypes.c_int32),
        ("n_classes", ctypes.c_int32),
        ("need_gcam", ctypes.c_int32),
        ("ctas", ctypes.c_int32),
        ("workspace", ctypes.c_void_p),
        ("workspace_bytes", ctypes.c_uint64),
        ("reserved", ctypes.c_int32 * 4),
    ]

    def __init__(self, **kw):
        super().__init__(**kw)
        self.struct_size = ctypes.sizeof(BatchArgs)
        self.abi_version = _ffi.ABI_VERSION


@dataclass
class RenderRequest:
    subject: object
    k_inv: torch.Tensor   # [1, 3, 3]
    sdd: torch.Tensor     # [1]
    height: int
    width: int
    n_samples: int = 500
    orthographic: bool = False


class BatchedRenderer:
    """Static-buffer batched renderer; see the module docstring."""

    def __init__(self, requests: list[RenderRequest], n_classes: int = 1, autotuner: Autotuner | None = None,
                 default_shape=(16, 16, 1), device=None, layout: str = "quad"):
        if not requests:
            raise ValueError("no requests")
        self.device = torch.device(device or requests[0].subject.image.device)
        self.C = n_classes
        vols = [r.subject.image[0, 0].contiguous() for r in requests]
        dt = vols[0].dtype
        if any(v.dtype != dt for v in vols):
            raise ValueError("all volumes of a batch must share one dtype")
        self.dtype = dt
        self.requests = requests
        R = len(requests)
        # camera-space rays: pose independent, computed once
        self.src, self.tgt, self.step = [], [], []
        for r in requests:
            src, tgt = _camera_rays(r.k_inv, r.sdd, r.height, r.width, r.orthographic, self.device, torch.float32)
            src, tgt = src.contiguous(), tgt.contiguous()
            step = ((tgt - src).norm(dim=-1) / (r.n_samples - 1)).contiguous()
            self.src.append(src)
            self.tgt.append(tgt)
            self.step.append(step)
        self.N = [r.height * r.width for r in requests]
        # static buffers
        self.M = torch.zeros(R, 3, 4, device=self.device)
        self.gM = torch.zeros(R, 3, 4, device=self.device)
        self.gsrc = [torch.zeros(s.shape[1:], device=self.device) for s in self.src]
        self.offsets = np.concatenate([[0], np.cumsum([n * self.C for n in self.N])])
        self.out_flat = torch.empty(int(self.offsets[-1]), device=self.device, dtype=dt)
        self.go_flat = torch.zeros(int(self.offsets[-1]), device=self.device, dtype=dt)
        self.w2v = torch.stack([r.subject.world_to_voxel.float()[:3] for r in requests]).to(self.device)
        self.labs = [compact_label(r.subject) if n_classes > 1 else v for r, v in zip(requests, vols)]
        self.vols = vols
        if layout not in ("quad", "plain"):
            raise ValueError(f"layout must be 'quad' or 'plain', got {layout!r}")
        # one quad-layout copy per distinct subject (cached on the subject)
        self.quads = [cached_quad(r.subject, v) if layout == "quad" else None for r, v in zip(requests, vols)]
        # launch shapes
        shapes = []
        for i, r in enumerate(requests):
            if autotuner is None:
                shapes.append(tuple(default_shape))
            else:
                shapes.append(autotuner.best_shape(
                    vols[i], self.labs[i], self._center_pose_M(i)[None].contiguous(),
                    self.src[i], self.tgt[i], self.step[i], r.n_samples, n_classes, r.width,
                    candidates=BATCHED_CANDIDATES, quad=self.quads[i],
                ))
        self.shapes = shapes
        # work order: most expensive first
        cost = [self.N[i] * requests[i].n_samples for i in range(R)]
        self.order = sorted(range(R), key=lambda i: -cost[i])
        self._build_descriptors()

    def _center_pose_M(self, i):
        """A representative camera->voxel affine for tuning: the identity AP
        pose with the source 600 mm from the isocenter."""
        from .phantom import identity_pose

        rt = identity_pose().to(self.device)
        return _affine_product(self.w2v[i], rt)[0]

    def _build_descriptors(self):
        R = len(self.requests)
        arr = (Request * R)()
        es = self.out_flat.element_size()
        for slot, i in enumerate(self.order):
            r = self.requests[i]
            q = arr[slot]
            q.vol = self.vols[i].data_ptr()
            q.lab = self.labs[i].data_ptr() if self.C > 1 else None
            q.D, q.H, q.W = self.vols[i].shape
            q.N, q.width, q.n_samples = self.N[i], r.width, r.n_samples
            q.src_per_ray = 0 if self.src[i].shape[1] == 1 else 1
            q.tile_w, q.tile_h, q.sample_split = self.shapes[i]
            q.M = self.M[i].data_ptr()
            q.src, q.tgt, q.step = self.src[i].data_ptr(), self.tgt[i].data_ptr(), self.step[i].data_ptr()
            q.out = self.out_flat.data_ptr() + int(self.offsets[i]) * es
            q.go = self.go_flat.data_ptr() + int(self.offsets[i]) * es
            q.gM = self.gM[i].data_ptr()
            q.gsrc = self.gsrc[i].data_ptr()
            q.vol_quad = self.quads[i].data_ptr() if self.quads[i] is not None else None
        tiles = (ctypes.c_int32 * R)()
        lib = _ffi.load()
        _ffi.check(lib.ndrr_batch_validate(arr, R, self.C, tiles), "ndrr_batch_validate")
        self.tiles = np.array(list(tiles), dtype=np.int64)
        off = np.concatenate([[0], np.cumsum(self.tiles)]).astype(np.int32)
        self.total_tiles = int(off[-1])
        raw = np.frombuffer(bytes(arr), dtype=np.uint8).copy()
        self.desc = torch.from_numpy(raw).to(self.device)
        self.tile_offsets = torch.from_numpy(off).to(self.device)
        nb = ctypes.c_uint64()
        _ffi.check(lib.ndrr_batched_workspace_bytes(self.total_tiles, ctypes.byref(nb)), "workspace")
        self.workspace = torch.empty(int(nb.value), dtype=torch.uint8, device=self.device)

    # ------------------------------------------------------------ execution
    def set_poses(self, rt_inv: torch.Tensor) -> None:
        """Camera-to-world poses [R, 4, 4] (request order) -> stacked M."""
        self.M.copy_((self.w2v[:, :, :, None] * rt_inv[:, None, :, :]).sum(dim=2))

    def _args(self, backward: bool) -> BatchArgs:
        a = BatchArgs()
        a.requests = self.desc.data_ptr()
        a.tile_offsets = self.tile_offsets.data_ptr()
        a.n_requests = len(self.requests)
        a.total_tiles = self.total_tiles
        a.vol_dtype = ndrr_dtype(self.vols[0])
        a.lab_dtype = ndrr_dtype(self.labs[0]) if self.C > 1 else 0
        a.go_dtype = ndrr_dtype(self.go_flat)
        a.n_classes = self.C
        a.need_gcam = 0
        a.workspace = self.workspace.data_ptr()
        a.workspace_bytes = self.workspace.numel()
        return a

    def forward(self) -> None:
        a = self._args(False)
        lib = _ffi.load()
        _ffi.check(lib.ndrr_batched_fwd(ctypes.byref(a), torch.cuda.current_stream(self.device).cuda_stream),
                   "ndrr_batched_fwd")

    def backward(self) -> None:
        """Pose adjoint of `go_flat` into gM (per request [3, 4])."""
        a = self._args(True)
        lib = _ffi.load()
        _ffi.check(lib.ndrr_batched_bwd(ctypes.byref(a), torch.cuda.current_stream(self.device).cuda_stream),
                   "ndrr_batched_bwd")

    def output(self, i: int) -> torch.Tensor:
        r = self.requests[i]
        return self.out_flat[int(self.offsets[i]) : int(self.offsets[i + 1])].view(self.C, r.height, r.width)

    def go(self, i: int) -> torch.Tensor:
        r = self.requests[i]
        return self.go_flat[int(self.offsets[i]) : int(self.offsets[i + 1])].view(self.C, r.height, r.width)

    def pose_grad(self) -> torch.Tensor:
        """dL/d rt_inv [R, 4, 4] from gM (rows 0..3; M = world_to_voxel[:3] @ rt_inv)."""
        return torch.einsum("rij,rik->rjk", self.w2v, self.gM)
