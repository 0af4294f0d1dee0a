"""CPU oracle for the ray-march path — TEST INFRASTRUCTURE ONLY.

Only `tests/`, `__graft_entry__.smoke()` and the CPU-baseline leg of
`bench.py` import this package, and only as the checker / the reported CPU
baseline. The product (`nanodrr_gb300`) never imports it.

Two independent restatements of the reference renderer:
  - `render_oracle` (grid_oracle.py): the reference's PyTorch backend
    `render_torch` (nanodrr src/nanodrr/drr/backends.py:9-63) — normalised-grid
    transform, linspace samples, grid_sample bilinear/nearest with zero
    padding, Riemann sum × step, scatter into label channels — run on CPU in
    any dtype (float64 for the FP64 oracle); autograd through grid_sample is the
    reference's analytic backward for that backend.
  - `march_numpy` / `march_numpy_adjoint` (numpy_oracle.py): the per-sample
    arithmetic of the reference's fused kernel (src/nanodrr/drr/_fused.py:133-
    298) in float64 numpy, with the analytic adjoint, used to pin the
    voxel-index formulation against the grid formulation and for central
    finite-difference checks.

Parity pin: both restatements are checked against golden fixtures produced by
the reference itself (`tests/golden/make_golden.py`, run in a container where
the reference imports) — see tests/test_oracle.py.
"""

from .grid_oracle import make_src, make_tgt, render_oracle, render_oracle_chunked, voxel_to_grid
from .homography_oracle import resample_oracle, resample_pixels
from .ncc_oracle import ncc_oracle
from .numpy_oracle import march_numpy, march_numpy_adjoint

__all__ = [
    "ncc_oracle",
    "resample_oracle",
    "resample_pixels",
    "make_src",
    "make_tgt",
    "render_oracle",
    "render_oracle_chunked",
    "voxel_to_grid",
    "march_numpy",
    "march_numpy_adjoint",
]
