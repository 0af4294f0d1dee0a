"""The C-ABI library builds, loads and exports every symbol its header declares,
and its host-side validation rejects bad arguments with the documented status
codes — all without a GPU (no call here launches a kernel)."""

import ctypes
import re
from pathlib import Path

import pytest

from nanodrr_gb300 import _build, _ffi

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared_symbols() -> set[str]:
    names = set()
    for h in HEADERS:
        for m in re.finditer(r"NDRR_API\s+[\w\s\*]+?\b(ndrr_\w+)\s*\(", h.read_text()):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _ffi.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"ndrr_raymarch_fwd", "ndrr_raymarch_bwd", "ndrr_raymarch_bwd_workspace_bytes", "ndrr_last_error"} <= names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert set(_ffi.SIGNATURES) >= declared_symbols()


def test_abi_version_and_struct_layout(lib):
    assert lib.ndrr_abi_version() == _ffi.ABI_VERSION
    assert b"sm_103a" in lib.ndrr_build_info()
    # 64-bit layout of ndrr_raymarch_args as declared in the header
    assert ctypes.sizeof(_ffi.RaymarchArgs) == 360
    assert ctypes.sizeof(_ffi.OccupancyArgs) == 56


def _valid_args():
    a = _ffi.RaymarchArgs()
    a.vol = 0x1000
    a.vol_dtype = _ffi.NDRR_F32
    a.D, a.H, a.W = 8, 8, 8
    a.n_classes = 1
    a.M = a.src = a.tgt = a.step = 0x2000
    a.B, a.N, a.width, a.n_samples = 2, 64, 8, 16
    a.out = 0x3000
    return a


def test_workspace_query_needs_no_gpu(lib):
    a = _valid_args()
    nb = ctypes.c_uint64()
    assert lib.ndrr_raymarch_bwd_workspace_bytes(ctypes.byref(a), ctypes.byref(nb)) == _ffi.NDRR_OK
    # 8 x 8 image of a small launch: default 8 x 4 tiles -> 2 tiles per pose,
    # 16 floats per tile
    assert nb.value == 2 * 2 * 16 * 4
    a.tile_w, a.tile_h = 16, 8  # a chosen tile: 1 tile per pose
    assert lib.ndrr_raymarch_bwd_workspace_bytes(ctypes.byref(a), ctypes.byref(nb)) == _ffi.NDRR_OK
    assert nb.value == 2 * 1 * 16 * 4


@pytest.mark.parametrize(
    "field,value,code,needle",
    [
        ("n_samples", 1, _ffi.NDRR_ERR_INVALID_ARGUMENT, "n_samples"),
        ("vol_dtype", _ffi.NDRR_U8, _ffi.NDRR_ERR_DTYPE, "volume dtype"),
        ("D", 0, _ffi.NDRR_ERR_INVALID_ARGUMENT, "dims"),
        ("vol", None, _ffi.NDRR_ERR_INVALID_ARGUMENT, "vol is NULL"),
        ("n_classes", 0, _ffi.NDRR_ERR_INVALID_ARGUMENT, "n_classes"),
        ("n_classes", 3, _ffi.NDRR_ERR_INVALID_ARGUMENT, "label map"),
        ("tile_w", 12, _ffi.NDRR_ERR_INVALID_ARGUMENT, "tile_w"),
        ("sample_split", 3, _ffi.NDRR_ERR_INVALID_ARGUMENT, "sample_split"),
        ("struct_size", 8, _ffi.NDRR_ERR_INVALID_ARGUMENT, "struct_size"),
        ("out", None, _ffi.NDRR_ERR_INVALID_ARGUMENT, "out is NULL"),
        ("tgt", None, _ffi.NDRR_ERR_INVALID_ARGUMENT, "non-NULL"),
    ],
)
def test_forward_rejects_bad_arguments(lib, field, value, code, needle):
    a = _valid_args()
    setattr(a, field, value)
    rc = lib.ndrr_raymarch_fwd(ctypes.byref(a), None)
    assert rc == code
    assert needle in lib.ndrr_last_error().decode()


def test_int32_limits_rejected(lib):
    a = _valid_args()
    a.D, a.H, a.W = 2048, 1024, 1024  # 2^31 voxels
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_LIMIT
    a = _valid_args()
    a.B, a.N = 65536, 65536
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_LIMIT


def test_empty_batch_is_a_no_op(lib):
    a = _valid_args()
    a.B = 0
    a.M = a.src = a.tgt = a.step = None
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_OK


def test_backward_rejects_missing_outputs_and_workspace(lib):
    a = _valid_args()
    a.go = 0x4000
    a.go_dtype = _ffi.NDRR_F32
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT  # gM NULL
    a.gM = 0x5000
    a.need_gvol = 1
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT  # gvol NULL
    a.need_gvol = 0
    a.need_gcam = 1
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT  # gsrc NULL
    a.need_gcam = 0
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_WORKSPACE
    a.workspace = 0x6000
    a.workspace_bytes = 8
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_WORKSPACE
    assert "workspace" in lib.ndrr_last_error().decode()


def test_status_codes_map_to_reference_exceptions(lib):
    a = _valid_args()
    a.n_samples = 1
    with pytest.raises(ValueError, match="n_samples"):
        _ffi.check(lib.ndrr_raymarch_fwd(ctypes.byref(a), None), "fwd")
    with pytest.raises(RuntimeError):
        _ffi.check(_ffi.NDRR_ERR_CUDA, "fwd")


def test_batch_validation_is_host_only_and_counts_tiles(lib):
    from nanodrr_gb300.batched import BatchArgs, Request

    assert ctypes.sizeof(Request) == 144
    assert ctypes.sizeof(BatchArgs) == 88
    arr = (Request * 2)()
    for q, (n, w) in zip(arr, ((256 * 256, 256), (200 * 200, 200))):
        q.vol = q.M = q.src = q.tgt = q.step = 0x1000
        q.D = q.H = q.W = 64
        q.N, q.width, q.n_samples = n, w, 100
        q.tile_w, q.tile_h, q.sample_split = 16, 16, 1
    tiles = (ctypes.c_int32 * 2)()
    assert lib.ndrr_batch_validate(arr, 2, 1, tiles) == _ffi.NDRR_OK
    assert list(tiles) == [16 * 16, 13 * 13]
    arr[1].sample_split = 2  # 16 x 16 x 2 != 256 threads
    assert lib.ndrr_batch_validate(arr, 2, 1, tiles) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "request 1" in lib.ndrr_last_error().decode()
    nb = ctypes.c_uint64()
    assert lib.ndrr_batched_workspace_bytes(100, ctypes.byref(nb)) == 0 and nb.value == 256 + 100 * 64


def test_sample_window_rules_are_host_only(lib):
    a = _valid_args()
    a.sample_window = 0x7004  # not 8-byte aligned
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "aligned" in lib.ndrr_last_error().decode()
    a.sample_window = 0x7000
    a.skip_mode = _ffi.NDRR_SKIP_OCCUPANCY
    a.occ_grid, a.occ_cell = 0x8000, 4
    a.occ_gx = a.occ_gy = a.occ_gz = 4
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "exclusive" in lib.ndrr_last_error().decode()
    b = _valid_args()
    b.sample_window = 0x7000
    b.go, b.go_dtype, b.gM = 0x4000, _ffi.NDRR_F32, 0x5000
    b.need_gvol, b.gvol = 1, 0x9000
    assert lib.ndrr_raymarch_bwd(ctypes.byref(b), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "every sample" in lib.ndrr_last_error().decode()


def test_skip_windows_validation(lib):
    a = _valid_args()
    assert lib.ndrr_skip_windows(ctypes.byref(a), 0x7000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT  # no skip mode
    a.skip_mode = _ffi.NDRR_SKIP_OCCUPANCY
    a.occ_grid, a.occ_cell = 0x8000, 4
    a.occ_gx = a.occ_gy = a.occ_gz = 4
    assert lib.ndrr_skip_windows(ctypes.byref(a), None, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "windows is NULL" in lib.ndrr_last_error().decode()
    assert lib.ndrr_skip_windows(ctypes.byref(a), 0x7002, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT


def test_pose_entry_points_validate_on_the_host(lib):
    """ndrr_pose_so3_fwd/bwd: NULL inputs and a parameter row count other
    than 1 or B are rejected before any launch; B = 0 is a no-op."""
    p = 0x7000  # never dereferenced: validation fails or returns first
    f, b = lib.ndrr_pose_so3_fwd, lib.ndrr_pose_so3_bwd
    assert f(None, p, 1, p, p, p, 4, p, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert f(p, p, 3, p, p, p, 4, p, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "param_rows" in lib.ndrr_last_error().decode()
    assert f(p, p, 1, p, p, p, 4, None, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert f(p, p, 1, p, p, p, -1, p, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert f(None, None, 1, None, None, None, 0, None, None) == _ffi.NDRR_OK
    assert b(p, p, p, 4, p, p, p, 4, None, p, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert b(None, p, p, 4, p, p, p, 4, p, p, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert b(p, p, p, 2, p, p, p, 4, p, p, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert b(None, None, None, 1, None, None, None, 0, None, None, None) == _ffi.NDRR_OK


@pytest.mark.parametrize("field,addr,expect", [
    ("vol_quad", 0x7008, "vol_quad"),
    ("gvol_quad", 0x7004, "gvol_quad"),
    ("gvol", 0x9004, "gvol"),
    ("M", 0x2002, "M"),
    ("workspace", 0x6008, "workspace"),
])
def test_misaligned_pointers_are_refused_before_any_launch(lib, field, addr, expect):
    """Pointers the kernels access with 16-byte vector instructions (quad
    layout, its gradient scratch, the volume gradient the quad fold writes,
    the workspace) and every element pointer must be aligned; a C caller
    passing an offset view gets NDRR_ERR_INVALID_ARGUMENT, not a GPU fault."""
    a = _valid_args()
    a.vol_quad = 0x7000
    a.go, a.go_dtype, a.gM = 0x4000, _ffi.NDRR_F32, 0x5000
    a.need_gvol, a.gvol, a.gvol_quad = 1, 0x9000, 0x7000
    a.workspace, a.workspace_bytes = 0x6000, 1 << 30
    setattr(a, field, addr)
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    msg = lib.ndrr_last_error().decode()
    assert expect in msg and "aligned" in msg
    nbytes = ctypes.c_uint64(0)
    assert lib.ndrr_raymarch_bwd_workspace_bytes(ctypes.byref(a), ctypes.byref(nbytes)) == \
        _ffi.NDRR_ERR_INVALID_ARGUMENT


def test_quad_build_and_hu_to_mu_validate_on_the_host(lib):
    assert lib.ndrr_quad_build(0x1000, _ffi.NDRR_F32, 4, 4, 4, 0x2008, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_hu_to_mu(0x1000, _ffi.NDRR_F32, -1, 0.02, 0.05, 1000.0, 0x1000, None) == \
        _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_hu_to_mu(0x1000, _ffi.NDRR_U8, 4, 0.02, 0.05, 1000.0, 0x1000, None) == _ffi.NDRR_ERR_DTYPE
    assert lib.ndrr_hu_to_mu(None, _ffi.NDRR_F32, 0, 0.02, 0.05, 1000.0, None, None) == _ffi.NDRR_OK


def test_measurement_entry_points_validate_on_the_host(lib):
    assert lib.ndrr_set_kernel_events(0x1000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_set_kernel_events(None, None) == _ffi.NDRR_OK
    assert lib.ndrr_l2_read_probe(None, 1024, 1, 0x2000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_l2_read_probe(0x1008, 1024, 1, 0x2000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_l2_read_probe(0x1000, 1024, 0, 0x2000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    flags = ctypes.c_uint32(0)
    assert lib.ndrr_device_flags(None, 0) == _ffi.NDRR_ERR_INVALID_ARGUMENT


def test_labelled_quad_validates_on_the_host(lib):
    a = _valid_args()
    a.vol_quad, a.quad_labels = 0x7000, 1  # f32 volume: not for the labelled layout
    a.n_classes, a.lab, a.lab_dtype = 3, 0x6000, _ffi.NDRR_U8
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "labelled" in lib.ndrr_last_error().decode()
    a.vol_dtype, a.n_classes = _ffi.NDRR_BF16, 1  # one channel: no labels to carry
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    a.quad_labels, a.vol_quad = 1, None
    assert lib.ndrr_raymarch_fwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    b = lib.ndrr_quad_build_labeled
    assert b(0x1000, _ffi.NDRR_F32, 0x2000, _ffi.NDRR_U8, 3, 4, 4, 4, 0x3000, None) == _ffi.NDRR_ERR_DTYPE
    assert b(0x1000, _ffi.NDRR_BF16, 0x2000, _ffi.NDRR_U8, 1, 4, 4, 4, 0x3000, None) == \
        _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert b(0x1000, _ffi.NDRR_BF16, 0x2000, _ffi.NDRR_U8, 3, 4, 4, 4, 0x3008, None) == \
        _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert b(0x1000, _ffi.NDRR_BF16, None, _ffi.NDRR_U8, 3, 4, 4, 4, 0x3000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT


def test_camera_rays_validate_on_the_host(lib):
    r = lib.ndrr_camera_rays
    assert r(None, 1, 0x2000, 1, 1, 4, 4, 0, 0x3000, 0x4000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert r(0x1000, 1, 0x2000, 1, 1, 0, 4, 0, 0x3000, 0x4000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert r(0x1000, 2, 0x2000, 3, 3, 4, 4, 0, 0x3000, 0x4000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert r(0x1000, 1, 0x2000, 1, 2, 4, 4, 0, 0x3000, 0x4000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert r(0x1000, 1, 0x2000, 1, 1, 4, 4, 0, 0x3002, 0x4000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert r(0x1000, 1, 0x2000, 1, 40000, 200, 200, 0, 0x3000, 0x4000, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert r(0x1000, 40000, 0x2000, 1, 40000, 200, 200, 0, 0x3000, 0x4000, None) == _ffi.NDRR_ERR_LIMIT


def test_split_adjoint_rules_are_host_only(lib):
    """Sample windows with a volume gradient: taken by the slab-ordered
    adjoint of one channel (as gather windows) and by gvol_mode 5 (its pose
    pass), refused by the direct scatter; mode 5 needs the quad layout;
    modes above 5 are refused."""
    a = _valid_args()
    a.go, a.go_dtype, a.gM = 0x4000, _ffi.NDRR_F32, 0x5000
    a.need_gvol, a.gvol = 1, 0x8000
    a.sample_window = 0x9000
    a.gvol_mode = _ffi.NDRR_GVOL_DIRECT
    a.vol_quad, a.gvol_quad = 0xA000, 0xB000
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert "gvol_mode 5" in lib.ndrr_last_error().decode()
    a.gvol_mode = _ffi.NDRR_GVOL_SLAB
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_WORKSPACE  # windows accepted
    a.gvol_mode = _ffi.NDRR_GVOL_SPLIT
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_WORKSPACE  # windows accepted
    a.vol_quad = None
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    a.vol_quad, a.gvol_mode = 0xA000, 6
    assert lib.ndrr_raymarch_bwd(ctypes.byref(a), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT


def test_reduction_probe_validates_on_the_host(lib):
    n = ctypes.c_int32(0)
    plane = 512 * 512 * 16
    assert lib.ndrr_reduce_probe(None, 5 * plane, 1, ctypes.byref(n), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_reduce_probe(0x1008, 5 * plane, 1, ctypes.byref(n), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_reduce_probe(0x1000, 4 * plane, 1, ctypes.byref(n), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_reduce_probe(0x1000, 5 * plane, 0, ctypes.byref(n), None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
    assert lib.ndrr_reduce_probe(0x1000, 5 * plane, 1, None, None) == _ffi.NDRR_ERR_INVALID_ARGUMENT
