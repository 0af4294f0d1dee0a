"""The allocation-free adjoint entry point (`ndrr_raymarch_bwd_noalloc`).

It exists for callers that cannot allocate device memory where they run the
adjoint — hosts that own all device memory through their own pool, and
real-time loops that cannot afford a cudaMalloc — and keeps its scratch in a
fixed array inside the library. Called through the C ABI, it must give the
same gradients as `ndrr_raymarch_bwd` with a caller workspace, on two calls
in a row (the shared scratch keeps the previous call's contents), and must
reject calls whose scratch would not fit. This file is collected last.
"""

import ctypes

import numpy as np
import pytest
import torch

from nanodrr_gb300 import _build, _ffi

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _args(seed, B=3, Hd=24, Wd=40, shape=(30, 34, 38), n=150):
    """Device buffers and a filled ndrr_raymarch_args for a small adjoint."""
    rng = np.random.default_rng(seed)
    D, H, W = shape
    vol = torch.from_numpy(rng.random(shape).astype(np.float32)).to(DEV)
    M = np.zeros((B, 3, 4), np.float32)
    for b in range(B):
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        M[b, :, :3] = q
        M[b, :, 3] = np.array([W, H, D]) / 2 + rng.uniform(-2, 2, 3)
    N = Hd * Wd
    u, v = np.meshgrid(np.arange(Wd) - Wd / 2 + 0.5, np.arange(Hd) - Hd / 2 + 0.5)
    tgt = np.stack([u.ravel(), v.ravel(), np.full(N, 50.0)], -1)[None].repeat(B, 0).astype(np.float32)
    src = np.zeros((B, 1, 3), np.float32)
    src[..., 2] = -50.0
    step = (np.linalg.norm(tgt - src, axis=-1) / (n - 1)).astype(np.float32)
    t = {k: torch.from_numpy(x).to(DEV) for k, x in dict(M=M, src=src, tgt=tgt, step=step).items()}
    t["vol"] = vol
    t["go"] = torch.from_numpy(rng.standard_normal((B, 1, N)).astype(np.float32)).to(DEV)
    a = _ffi.RaymarchArgs()
    a.vol, a.vol_dtype, (a.D, a.H, a.W) = vol.data_ptr(), _ffi.NDRR_F32, shape
    a.n_classes = 1
    a.M, a.src, a.tgt, a.step = t["M"].data_ptr(), t["src"].data_ptr(), t["tgt"].data_ptr(), t["step"].data_ptr()
    a.src_per_ray, a.B, a.N, a.width, a.n_samples = 0, B, N, Wd, n
    a.go, a.go_dtype = t["go"].data_ptr(), _ffi.NDRR_F32
    a.need_gvol, a.need_gcam = 1, 1
    return a, t


def _outputs(a, t):
    B, N = a.B, a.N
    o = {
        "gvol": torch.zeros(a.D, a.H, a.W, device=DEV),
        "gM": torch.empty(B, 3, 4, device=DEV),
        "gsrc": torch.empty(B, 1, 3, device=DEV),
        "gtgt": torch.empty(B, N, 3, device=DEV),
        "gstep": torch.empty(B, N, device=DEV),
    }
    for k, v in o.items():
        setattr(a, k, v.data_ptr())
    return o


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_noalloc_adjoint_matches_workspace_adjoint_twice():
    _build.build()
    lib = _ffi.load()
    for seed in (0, 1):  # two different problems back to back share the scratch
        a, t = _args(seed)
        ref = _outputs(a, t)
        nb = ctypes.c_uint64()
        assert lib.ndrr_raymarch_bwd_workspace_bytes(ctypes.byref(a), ctypes.byref(nb)) == 0
        ws = torch.empty(nb.value, dtype=torch.uint8, device=DEV)
        a.workspace, a.workspace_bytes = ws.data_ptr(), ws.numel()
        assert lib.ndrr_raymarch_bwd(ctypes.byref(a), _stream()) == 0, lib.ndrr_last_error()
        for call in range(2):
            got = _outputs(a, t)
            a.workspace, a.workspace_bytes = None, 0
            rc = lib.ndrr_raymarch_bwd_noalloc(ctypes.byref(a), _stream())
            assert rc == 0, lib.ndrr_last_error()
            torch.cuda.synchronize()
            for k in ref:
                scale = ref[k].abs().max().clamp_min(1e-30)
                err = float((got[k] - ref[k]).abs().max() / scale)
                tol = 0.0 if k == "gM" else 1e-5  # pose partials: same order; gvol: atomics
                assert err <= tol, (seed, call, k, err)


def test_noalloc_adjoint_rejects_oversized_calls():
    _build.build()
    lib = _ffi.load()
    # 33 poses of 256 x 256 rays with 8 x 4 tiles: 33 * 2048 * 64 B > 4 MiB
    B, N = 33, 256 * 256
    z = torch.zeros(B * N * 3, device=DEV)
    vol = torch.zeros(8, 8, 8, device=DEV)
    a = _ffi.RaymarchArgs()
    a.vol, a.vol_dtype, a.D, a.H, a.W = vol.data_ptr(), _ffi.NDRR_F32, 8, 8, 8
    a.n_classes = 1
    a.M = a.src = a.tgt = a.step = a.go = a.gM = z.data_ptr()
    a.go_dtype = _ffi.NDRR_F32
    a.B, a.N, a.width, a.n_samples = B, N, 256, 16
    a.tile_w, a.tile_h = 8, 4
    rc = lib.ndrr_raymarch_bwd_noalloc(ctypes.byref(a), _stream())
    assert rc == _ffi.NDRR_ERR_LIMIT
    assert "allocation-free" in lib.ndrr_last_error().decode()
