"""nanodrr_gb300: differentiable DRR rendering on GB300 (sm_103a).

A drop-in for the fused backend of nanodrr's `render` call: the same inputs
(subject volume and optional label map, intrinsics, extrinsics, per-label
channels) and autograd through pose, intrinsics and volume, computed by
hand-written CUDA kernels behind a C ABI (`include/nanodrr_gb300.h`).
"""

from ._build import build
from .drr import DRR
from .geometry import convert, make_k_inv, make_rt_inv, transform_point
from .homography import resample
from .raymarch import fused_raymarch, fused_raymarch_bwd, raymarch_backward, raymarch_forward
from .renderer import fused_supported, render
from .subject import Subject, hu_to_mu

__all__ = [
    "resample",
    "build",
    "DRR",
    "Subject",
    "hu_to_mu",
    "render",
    "fused_supported",
    "fused_raymarch",
    "fused_raymarch_bwd",
    "raymarch_forward",
    "raymarch_backward",
    "convert",
    "make_k_inv",
    "make_rt_inv",
    "transform_point",
]
