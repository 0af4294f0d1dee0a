"""`DRR` module: cached detector geometry around `render`.

Mirrors the reference's `DRR` (nanodrr src/nanodrr/drr/drr.py:9-106):
`k_inv` and `sdd` are persistent buffers, the ray endpoints `src`/`tgt` are
non-persistent buffers recomputed whenever an intrinsic changes.
"""

from __future__ import annotations

import torch

from .geometry import make_k_inv
from .renderer import _make_src, _make_tgt, render


class DRR(torch.nn.Module):
    _intrinsic_params = {"k_inv", "sdd", "height", "width", "orthographic"}

    def __init__(self, k_inv: torch.Tensor, sdd: torch.Tensor, height: int, width: int, orthographic: bool = False):
        super().__init__()
        self.register_buffer("k_inv", k_inv)
        self.register_buffer("sdd", sdd)
        self.height = height
        self.width = width
        self.orthographic = orthographic
        self._compute_src_tgt()

    def __setattr__(self, name, value):
        super().__setattr__(name, value)
        if name in self._intrinsic_params and all(hasattr(self, p) for p in self._intrinsic_params):
            self._compute_src_tgt()

    def _compute_src_tgt(self):
        tgt = _make_tgt(self.k_inv, self.sdd, self.height, self.width, self.k_inv.device, self.k_inv.dtype)
        src = _make_src(self.orthographic, tgt, self.sdd)
        self.register_buffer("tgt", tgt, persistent=False)
        self.register_buffer("src", src, persistent=False)

    def forward(self, subject, rt_inv: torch.Tensor, n_samples: int = 500, backend: str = "auto"):
        return render(
            subject,
            self.k_inv,
            rt_inv,
            self.sdd,
            self.height,
            self.width,
            n_samples,
            self.orthographic,
            self.src,
            self.tgt,
            backend,
        )

    @classmethod
    def from_carm_intrinsics(
        cls, sdd, delx, dely, x0, y0, height, width, orthographic=False, dtype=None, device=None
    ) -> "DRR":
        k_inv = make_k_inv(sdd, delx, dely, x0, y0, height, width).to(dtype=dtype, device=device)
        return cls(k_inv, torch.tensor([sdd], dtype=dtype, device=device), height, width, orthographic)
