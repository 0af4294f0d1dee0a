"""`DRR` module: a detector (intrinsics, size, projection) that renders a
subject at given poses.

Interface of the reference's `DRR` (nanodrr src/nanodrr/drr/drr.py:9-106):
the constructor, `k_inv` and `sdd` as buffers (moved by `.to()`, saved in the
state dict), plain `height` / `width` / `orthographic` attributes, readable
camera-space ray endpoints `src` and `tgt`, `forward(subject, rt_inv,
n_samples, backend)` and `from_carm_intrinsics`.

The ray endpoints are derived data, not state: they are built on first use
from the current intrinsics and kept with a record of what they were built
from (the `k_inv` and `sdd` tensor objects by weak reference, their version
counters, the detector size and the projection). Reassigning any of these,
editing `k_inv` or `sdd` in place, or moving the module makes the record
stale and the next read rebuilds the rays, so no attribute hook is needed.
When `k_inv` or `sdd` requires a gradient the rays are rebuilt on every
read, so each forward has its own autograd graph. `forward` leaves the ray
construction to `render`, which keeps its own cache of the same rays keyed
the same way.
"""

from __future__ import annotations

import weakref

import torch

from .geometry import make_k_inv
from .renderer import _camera_rays, render


class DRR(torch.nn.Module):
    def __init__(self, k_inv: torch.Tensor, sdd: torch.Tensor, height: int, width: int, orthographic: bool = False):
        super().__init__()
        self.register_buffer("k_inv", k_inv)
        self.register_buffer("sdd", sdd)
        self.height = height
        self.width = width
        self.orthographic = orthographic
        self._ray_record = None  # (what the rays were built from, (src, tgt))

    def _ray_source(self) -> tuple:
        k, s = self.k_inv, self.sdd
        return (k._version, s._version, int(self.height), int(self.width), bool(self.orthographic))

    def rays(self) -> tuple[torch.Tensor, torch.Tensor]:
        """Camera-space ray endpoints (src [B, 1 | H*W, 3], tgt [B, H*W, 3])
        of the current intrinsics."""
        k, s = self.k_inv, self.sdd
        rec = self._ray_record
        if rec is not None:
            kref, sref, source, built = rec
            if kref() is k and sref() is s and source == self._ray_source():
                return built
        built = _camera_rays(k, s, int(self.height), int(self.width), bool(self.orthographic), k.device, k.dtype)
        if not (k.requires_grad or s.requires_grad):
            self._ray_record = (weakref.ref(k), weakref.ref(s), self._ray_source(), built)
        return built

    @property
    def src(self) -> torch.Tensor:
        return self.rays()[0]

    @property
    def tgt(self) -> torch.Tensor:
        return self.rays()[1]

    def forward(self, subject, rt_inv: torch.Tensor, n_samples: int = 500, backend: str = "auto") -> torch.Tensor:
        """[B, C, H, W] DRR of `subject` at the camera-to-world poses `rt_inv`."""
        return render(subject, self.k_inv, rt_inv, self.sdd, int(self.height), int(self.width), n_samples,
                      bool(self.orthographic), backend=backend)

    @classmethod
    def from_carm_intrinsics(
        cls, sdd, delx, dely, x0, y0, height, width, orthographic=False, dtype=None, device=None
    ) -> "DRR":
        """Detector of a C-arm: source-to-detector distance `sdd` (mm), pixel
        spacings `delx`, `dely` (mm), principal-point offsets `x0`, `y0` (mm)
        and the detector size in pixels."""
        placed = dict(dtype=dtype, device=device)
        k_inv = make_k_inv(sdd, delx, dely, x0, y0, height, width).to(**placed)
        return cls(k_inv, torch.full((1,), float(sdd), **placed), height, width, orthographic)
