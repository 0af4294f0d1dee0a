"""Launch-shape autotuner for the ray-march kernels.

The reference uses fixed tiling constants (nanodrr src/nanodrr/drr/_fused.py:
5-7) and a split heuristic (`_split`, :341-346). Here the tile shape and the
in-CTA sample split, and the slab size of the slab-ordered volume-gradient
adjoint, are picked per request class by timing candidates on the caller's
own rays with CUDA events, and cached (in memory and, when a path is given,
in a JSON file) under a key of volume shape, dtype, detector, sample count,
classes and batch size.
"""

from __future__ import annotations

import json
import os
import statistics
from pathlib import Path

import torch

from .raymarch import raymarch_backward, raymarch_forward

# (tile_w, tile_h, sample_split) with 256 threads: the batched kernel's shapes.
BATCHED_CANDIDATES = [(16, 16, 1), (16, 8, 2), (8, 8, 4), (32, 8, 1)]
# shapes for the single-request kernels (up to 512 threads)
SINGLE_CANDIDATES = [(16, 8, 1), (16, 16, 1), (32, 8, 1), (16, 8, 2), (8, 8, 4), (16, 8, 4), (8, 4, 4), (8, 4, 8),
                     (8, 8, 8), (8, 4, 16)]
# quad-gradient MiB per slab for the slab-ordered volume-gradient adjoint
SLAB_CANDIDATES = [48, 96, 192]


class Autotuner:
    def __init__(self, path: str | os.PathLike | None = None, reps: int = 5):
        self.path = Path(path) if path is not None else None
        self.reps = reps
        self.cache: dict[str, list[int]] = {}
        if self.path is not None and self.path.exists():
            try:
                self.cache = json.loads(self.path.read_text())
            except (OSError, ValueError):
                self.cache = {}

    @staticmethod
    def key(vol, n_classes, B, N, width, n_samples, candidates) -> str:
        D, H, W = vol.shape
        tag = "b" if candidates is BATCHED_CANDIDATES else "s"
        return f"{tag}:{D}x{H}x{W}:{str(vol.dtype).split('.')[-1]}:C{n_classes}:B{B}:N{N}:w{width}:S{n_samples}"

    def _time(self, fn) -> float:
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(self.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    def best_shape(self, vol, lab, M, src, tgt, step, n_samples, n_classes, width,
                   candidates=SINGLE_CANDIDATES, quad=None) -> tuple[int, int, int]:
        """Fastest (tile_w, tile_h, sample_split) for these rays (cached),
        timed on the quad layout when `quad` is given."""
        B, N, _ = tgt.shape
        k = self.key(vol, n_classes, B, N, width, n_samples, candidates) + (":q" if quad is not None else "")
        if k in self.cache:
            return tuple(self.cache[k])
        timings = {}
        for shape in candidates:
            timings[shape] = self._time(
                lambda: raymarch_forward(vol, lab, M, src, tgt, step, n_samples, n_classes, width, tile=shape,
                                         quad=quad)
            )
        best = min(timings, key=timings.get)
        self.cache[k] = list(best)
        self.save()
        return best

    def best_slab_mib(self, vol, quad, M, src, tgt, step, n_samples, width, n_classes=1, lab=None,
                      candidates=SLAB_CANDIDATES) -> int:
        """Fastest slab size (MiB of quad gradient) for the slab-ordered
        adjoint with volume gradient on these rays (cached); set it as
        `subject.slab_mib` for `render`."""
        B, N, _ = tgt.shape
        k = "slab:" + self.key(vol, n_classes, B, N, width, n_samples, None)
        if k in self.cache:
            return int(self.cache[k][0])
        lab = vol if lab is None else lab
        go = torch.ones(B, n_classes, N, device=vol.device)
        gvol = torch.zeros(vol.shape, device=vol.device)
        timings = {}
        for mib in candidates:
            timings[mib] = self._time(
                lambda: raymarch_backward(go, vol, lab, M, src, tgt, step, n_samples, n_classes, width, True, False,
                                          gvol=gvol, quad=quad, gvol_mode=3, slab_mib=mib)
            )
        best = min(timings, key=timings.get)
        self.cache[k] = [int(best)]
        self.save()
        return int(best)

    def save(self) -> None:
        if self.path is None:
            return
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            tmp = self.path.with_suffix(".tmp")
            tmp.write_text(json.dumps(self.cache, indent=1, sort_keys=True))
            os.replace(tmp, self.path)
        except OSError:
            pass
