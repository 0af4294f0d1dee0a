"""ctypes binding of the C ABI declared in `include/nanodrr_gb300.h`.

The library is loaded from the package's `_lib/` directory (built in-tree by
`nanodrr_gb300._build.build`). There is no fallback: if the library is missing
or fails to load, every render call raises.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

from . import _build

# ndrr_status
NDRR_OK = 0
NDRR_ERR_INVALID_ARGUMENT = 1
NDRR_ERR_LIMIT = 2
NDRR_ERR_DTYPE = 3
NDRR_ERR_WORKSPACE = 4
NDRR_ERR_CUDA = 5
NDRR_ERR_DEVICE_TIMEOUT = 6
NDRR_FLAG_TMA_TIMEOUT = 1

# ndrr_dtype
NDRR_F32, NDRR_F16, NDRR_BF16, NDRR_U8, NDRR_I8, NDRR_I16, NDRR_I32, NDRR_I64 = range(8)

ABI_VERSION = 3

# ndrr_gvol_mode
NDRR_GVOL_AUTO, NDRR_GVOL_DIRECT, NDRR_GVOL_BRICK, NDRR_GVOL_SLAB, NDRR_GVOL_SLAB_WARP, NDRR_GVOL_SPLIT = 0, 1, 2, 3, 4, 5

_c_float_p = ctypes.POINTER(ctypes.c_float)


class RaymarchArgs(ctypes.Structure):
    """Mirror of `ndrr_raymarch_args` (field order and types must match)."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("abi_version", ctypes.c_uint32),
        ("vol", ctypes.c_void_p),
        ("vol_dtype", ctypes.c_int32),
        ("D", ctypes.c_int32),
        ("H", ctypes.c_int32),
        ("W", ctypes.c_int32),
        ("lab", ctypes.c_void_p),
        ("lab_dtype", ctypes.c_int32),
        ("n_classes", ctypes.c_int32),
        ("M", ctypes.c_void_p),
        ("src", ctypes.c_void_p),
        ("tgt", ctypes.c_void_p),
        ("step", ctypes.c_void_p),
        ("src_per_ray", ctypes.c_int32),
        ("B", ctypes.c_int32),
        ("N", ctypes.c_int32),
        ("width", ctypes.c_int32),
        ("n_samples", ctypes.c_int32),
        ("t_window", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
        ("out_dtype", ctypes.c_int32),
        ("out_total", ctypes.c_void_p),
        ("go", ctypes.c_void_p),
        ("go_dtype", ctypes.c_int32),
        ("need_gvol", ctypes.c_int32),
        ("need_gcam", ctypes.c_int32),
        ("gvol", ctypes.c_void_p),
        ("gM", ctypes.c_void_p),
        ("gsrc", ctypes.c_void_p),
        ("gtgt", ctypes.c_void_p),
        ("gstep", ctypes.c_void_p),
        ("workspace", ctypes.c_void_p),
        ("workspace_bytes", ctypes.c_uint64),
        ("skip_mode", ctypes.c_int32),
        ("occ_cell", ctypes.c_int32),
        ("occ_gx", ctypes.c_int32),
        ("occ_gy", ctypes.c_int32),
        ("occ_gz", ctypes.c_int32),
        ("occ_grid", ctypes.c_void_p),
        ("proposal_params", ctypes.c_void_p),
        ("proposal_margin", ctypes.c_float),
        ("skip_stats", ctypes.c_void_p),
        ("out_extent", ctypes.c_void_p),
        ("vol_quad", ctypes.c_void_p),
        ("gvol_quad", ctypes.c_void_p),
        ("sample_window", ctypes.c_void_p),
        ("tile_w", ctypes.c_int32),
        ("tile_h", ctypes.c_int32),
        ("sample_split", ctypes.c_int32),
        ("gvol_mode", ctypes.c_int32),
        ("brick_cap", ctypes.c_int32),
        ("slab_mib", ctypes.c_int32),
        ("fwd_mode", ctypes.c_int32),
        ("gvol_overwrite", ctypes.c_int32),
        ("vol_texture", ctypes.c_uint64),
        ("quad_labels", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("M_lo", ctypes.c_void_p),
    ]

    def __init__(self, **kw):
        super().__init__(**kw)
        self.struct_size = ctypes.sizeof(RaymarchArgs)
        self.abi_version = ABI_VERSION


class OccupancyArgs(ctypes.Structure):
    """Mirror of `ndrr_occupancy_args`."""

    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("abi_version", ctypes.c_uint32),
        ("vol", ctypes.c_void_p),
        ("vol_dtype", ctypes.c_int32),
        ("D", ctypes.c_int32),
        ("H", ctypes.c_int32),
        ("W", ctypes.c_int32),
        ("cell", ctypes.c_int32),
        ("max_dist", ctypes.c_int32),
        ("grid", ctypes.c_void_p),
        ("scratch", ctypes.c_void_p),
    ]

    def __init__(self, **kw):
        super().__init__(**kw)
        self.struct_size = ctypes.sizeof(OccupancyArgs)
        self.abi_version = ABI_VERSION


# ndrr_skip_mode
NDRR_SKIP_NONE, NDRR_SKIP_OCCUPANCY, NDRR_SKIP_PROPOSAL = 0, 1, 2

_i32p = ctypes.POINTER(ctypes.c_int32)

# Every symbol the header declares, with its ctypes signature.
SIGNATURES: dict[str, tuple] = {
    "ndrr_abi_version": (ctypes.c_int32, []),
    "ndrr_build_info": (ctypes.c_char_p, []),
    "ndrr_last_error": (ctypes.c_char_p, []),
    "ndrr_device_flags": (ctypes.c_int32, [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int32]),
    "ndrr_raymarch_fwd": (ctypes.c_int32, [ctypes.POINTER(RaymarchArgs), ctypes.c_void_p]),
    "ndrr_raymarch_bwd_workspace_bytes": (
        ctypes.c_int32,
        [ctypes.POINTER(RaymarchArgs), ctypes.POINTER(ctypes.c_uint64)],
    ),
    "ndrr_raymarch_bwd": (ctypes.c_int32, [ctypes.POINTER(RaymarchArgs), ctypes.c_void_p]),
    "ndrr_raymarch_bwd_noalloc": (ctypes.c_int32, [ctypes.POINTER(RaymarchArgs), ctypes.c_void_p]),
    "ndrr_batch_validate": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "ndrr_batched_workspace_bytes": (ctypes.c_int32, [ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)]),
    "ndrr_batched_fwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_batched_bwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_quad_dims": (ctypes.c_int32, [ctypes.c_int32] * 3 + [_i32p] * 3),
    "ndrr_quad_build": (ctypes.c_int32, [ctypes.c_void_p] + [ctypes.c_int32] * 4 + [ctypes.c_void_p] * 2),
    "ndrr_quad_build_labeled": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
                                + [ctypes.c_int32] * 5 + [ctypes.c_void_p] * 2),
    "ndrr_camera_rays": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_hu_to_mu": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_set_kernel_events": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_l2_read_probe": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "ndrr_reduce_probe": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, _i32p, ctypes.c_void_p]),
    "ndrr_occupancy_dims": (ctypes.c_int32, [ctypes.c_int32] * 4 + [_i32p] * 3),
    "ndrr_occupancy_build": (ctypes.c_int32, [ctypes.POINTER(OccupancyArgs), ctypes.c_void_p]),
    "ndrr_skip_windows": (ctypes.c_int32, [ctypes.POINTER(RaymarchArgs), ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_texture_create": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]),
    "ndrr_texture_destroy": (ctypes.c_int32, [ctypes.c_uint64]),
    "ndrr_ncc_workspace_bytes": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_uint64)]),
    "ndrr_ncc_fwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_uint64, ctypes.c_void_p]),
    "ndrr_ncc_bwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_pose_so3_fwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "ndrr_pose_so3_bwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_homography_resample": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "ndrr_homography_resample_bwd_workspace_bytes": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                                      ctypes.POINTER(ctypes.c_uint64)]),
    "ndrr_homography_resample_bwd": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_uint64, ctypes.c_void_p]),
    "ndrr_proposal_last_error": (ctypes.c_char_p, []),
    "ndrr_proposal_dataset": (
        ctypes.c_int32,
        [ctypes.POINTER(RaymarchArgs), ctypes.c_void_p, ctypes.c_float] + [ctypes.c_void_p] * 4,
    ),
    "ndrr_proposal_train_step": (
        ctypes.c_int32,
        [ctypes.c_void_p] * 4 + [ctypes.c_int64, ctypes.c_float, ctypes.c_float] + [ctypes.c_void_p] * 3,
    ),
    "ndrr_proposal_forward": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 2),
    "ndrr_proposal_adam": (
        ctypes.c_int32,
        [ctypes.c_void_p] * 4 + [ctypes.c_int32] + [ctypes.c_float] * 4 + [ctypes.c_void_p],
    ),
    "ndrr_proposal_pack": (ctypes.c_int32, [ctypes.c_void_p] * 3),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def library_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the shared library and bind signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists() and build_if_missing:
            _build.build()
        if not path.exists():
            raise RuntimeError(f"nanodrr_gb300 CUDA library not found at {path}; run nanodrr_gb300.build()")
        lib = ctypes.CDLL(str(path))
        for name, (restype, argtypes) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        ver = lib.ndrr_abi_version()
        if ver != ABI_VERSION:
            raise RuntimeError(f"nanodrr_gb300 library ABI {ver} does not match the bindings' {ABI_VERSION}")
        _lib = lib
        return lib


class NdrrError(RuntimeError):
    pass


def check(rc: int, what: str) -> None:
    """Map a C-ABI status to the reference's exception types."""
    if rc == NDRR_OK:
        return
    msg = load().ndrr_last_error().decode(errors="replace")
    text = f"{what}: {msg}"
    if rc in (NDRR_ERR_INVALID_ARGUMENT, NDRR_ERR_LIMIT, NDRR_ERR_DTYPE):
        raise ValueError(text)
    raise NdrrError(text)
