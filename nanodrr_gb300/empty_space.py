"""Empty-space skipping for the ray march: occupancy grid and learned proposal.

Neither exists in the reference renderer, which marches every sample of each
ray's box-culled range (nanodrr src/nanodrr/drr/_fused.py:144-155, 190).

- `OccupancyGrid`: per-cell occupancy with a Chebyshev distance field, built
  on the GPU by `ndrr_occupancy_build`. A cell is occupied when any voxel
  within two voxels of it is non-zero, so a sample in an unoccupied cell has
  eight zero trilinear corners.
- `ProposalNetwork`: a 3-layer MLP (64-64-64-2, Fourier-encoded ray entry and
  exit points) that predicts where each ray's non-empty interval starts and
  ends. It is trained on the GPU by the project's own kernels
  (`ndrr_proposal_train_step`, `ndrr_proposal_adam`) on labels the plain
  renderer itself produces (its `extent` output: first and last sample with
  a non-zero corner), and packed to bf16 for the tensor-core inference of
  the window kernels (`ndrr_skip_windows`).
- `EmptySpace`: the configuration `render` reads from `subject.empty_space`.
  Mode "occupancy" marches each ray between the first and last occupied cell
  it crosses; mode "proposal" takes the network's interval when the grid
  confirms that nothing occupied lies outside it, and marches the full window
  otherwise (a fallback). Both leave the image and the pose/camera gradients
  unchanged; volume gradients always use the full window.
"""

from __future__ import annotations

import ctypes
import math
import weakref
from dataclasses import dataclass

import torch

from . import _ffi
from .raymarch import ndrr_dtype, raymarch_forward

PARAMS = 8450  # fp32 master parameters (W1, b1, W2, b2, W3, b3)
PACKED_BYTES = 17952
FEATURES = 64


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _root(t: torch.Tensor) -> torch.Tensor:
    """The tensor whose storage and version counter a view shares."""
    return t._base if t._base is not None else t


@dataclass
class OccupancyGrid:
    grid: torch.Tensor          # uint8 [gz, gy, gx] Chebyshev distance in cells (0 = occupied)
    cell: int
    volume_shape: tuple
    max_dist: int = 16
    # the volume the grid describes: (weak reference to its root tensor,
    # version counter, data pointer) at the last build
    source: tuple | None = None

    @classmethod
    def build(cls, vol: torch.Tensor, cell: int = 4, max_dist: int = 16) -> "OccupancyGrid":
        """Occupancy/distance grid of a [D, H, W] volume on its CUDA device."""
        if not vol.is_cuda or vol.dim() != 3:
            raise ValueError("vol must be a [D, H, W] CUDA tensor")
        g = cls(torch.empty(0, dtype=torch.uint8, device=vol.device), cell, tuple(vol.shape), max_dist)
        g._build(vol)
        return g

    def _build(self, vol: torch.Tensor) -> None:
        D, H, W = vol.shape
        lib = _ffi.load()
        gz, gy, gx = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _ffi.check(lib.ndrr_occupancy_dims(D, H, W, self.cell, ctypes.byref(gz), ctypes.byref(gy),
                                           ctypes.byref(gx)), "ndrr_occupancy_dims")
        shape = (gz.value, gy.value, gx.value)
        if tuple(self.grid.shape) != shape or self.grid.device != vol.device:
            self.grid = torch.empty(shape, dtype=torch.uint8, device=vol.device)
        scratch = torch.empty_like(self.grid)
        v = vol.detach().contiguous()
        a = _ffi.OccupancyArgs()
        a.vol, a.vol_dtype = v.data_ptr(), ndrr_dtype(v)
        a.D, a.H, a.W = D, H, W
        a.cell, a.max_dist = self.cell, self.max_dist
        a.grid, a.scratch = self.grid.data_ptr(), scratch.data_ptr()
        _ffi.check(lib.ndrr_occupancy_build(ctypes.byref(a), _stream(vol.device)), "ndrr_occupancy_build")
        self.volume_shape = (D, H, W)
        self.source = (weakref.ref(_root(vol)), vol._version, vol.data_ptr(), (D, H, W))

    def describes(self, vol: torch.Tensor) -> bool:
        """True when `vol` is the memory the grid was built from (the same
        tensor, a view or a detached alias of it) and has not changed since
        (version counter). While the tensor it was built from is alive that
        memory cannot belong to another volume; once it is gone, the grid
        is rebuilt."""
        if self.source is None:
            return False
        ref, version, ptr, shape = self.source
        if ref() is None:
            return False
        return vol.data_ptr() == ptr and tuple(vol.shape) == shape and vol._version == version

    def refresh(self, vol: torch.Tensor) -> bool:
        """Rebuild the grid (in place when the shape is unchanged) unless it
        describes `vol`; returns whether it rebuilt. Skipping with a grid of
        another volume, or of an earlier version of it, could drop samples
        that are no longer empty, so the render call refreshes first."""
        if self.describes(vol):
            return False
        self._build(vol)
        return True

    def occupied_fraction(self) -> float:
        return float((self.grid == 0).float().mean())


def _prop_check(rc: int, what: str) -> None:
    if rc != 0:
        msg = _ffi.load().ndrr_proposal_last_error().decode(errors="replace")
        raise (ValueError if rc in (1, 2, 3) else RuntimeError)(f"{what}: {msg}")


class ProposalNetwork:
    """fp32 master parameters, Adam state and the packed bf16 copy."""

    def __init__(self, device, seed: int = 0):
        self.device = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        p = torch.zeros(PARAMS)
        # He-style init for the ReLU layers, small output layer
        w1 = torch.randn(64, 64, generator=g) * math.sqrt(2.0 / 54)
        w1[:, 54:] = 0.0
        p[0:4096] = w1.flatten()
        p[4160:8256] = (torch.randn(64, 64, generator=g) * math.sqrt(2.0 / 64)).flatten()
        p[8320:8448] = (torch.randn(2, 64, generator=g) * 0.01).flatten()
        p[8448] = 0.0  # f_near bias: start wide (0 .. 1)
        p[8449] = 1.0
        self.params = p.to(self.device)
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.step = 0
        self.packed = torch.empty(PACKED_BYTES, dtype=torch.uint8, device=self.device)
        self.pack()

    # ---------------------------------------------------------------- data
    @staticmethod
    def dataset(vol, M, src, tgt, n_samples, width, extent, widen_voxels: float = 7.0):
        """(features [R, 64], targets [R, 2], valid [R]) for the rays of a
        batch of poses, from the plain renderer's `extent` output, each
        interval widened by `widen_voxels` (Chebyshev) so that the occupancy
        check (cell 4 + dilation) can confirm a correct prediction."""
        lib = _ffi.load()
        B, N, _ = tgt.shape
        a = _ffi.RaymarchArgs()
        a.D, a.H, a.W = vol.shape
        a.M, a.src, a.tgt = M.data_ptr(), src.data_ptr(), tgt.data_ptr()
        a.src_per_ray = 0 if src.shape[1] == 1 else 1
        a.B, a.N, a.width, a.n_samples = B, N, width, n_samples
        X = torch.empty(B * N, FEATURES, device=vol.device)
        T = torch.empty(B * N, 2, device=vol.device)
        V = torch.empty(B * N, dtype=torch.uint8, device=vol.device)
        _prop_check(
            lib.ndrr_proposal_dataset(ctypes.byref(a), ctypes.c_void_p(extent.data_ptr()),
                                      ctypes.c_float(widen_voxels),
                                      ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(T.data_ptr()),
                                      ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(_stream(vol.device))),
            "ndrr_proposal_dataset",
        )
        return X, T, V

    # ------------------------------------------------------------ training
    def train_step(self, X, T, V, alpha: float = 20.0, lr: float = 1e-3) -> torch.Tensor:
        """One Adam step on a minibatch; returns the loss (device scalar)."""
        lib = _ffi.load()
        grads = torch.zeros_like(self.params)
        loss = torch.zeros(1, device=self.device)
        n = X.shape[0]
        count = max(1, n)
        st = ctypes.c_void_p(_stream(self.device))
        _prop_check(
            lib.ndrr_proposal_train_step(
                ctypes.c_void_p(self.params.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(V.data_ptr()), ctypes.c_int64(n),
                ctypes.c_float(alpha), ctypes.c_float(1.0 / count), ctypes.c_void_p(grads.data_ptr()),
                ctypes.c_void_p(loss.data_ptr()), st,
            ),
            "ndrr_proposal_train_step",
        )
        self.step += 1
        _prop_check(
            lib.ndrr_proposal_adam(
                ctypes.c_void_p(self.params.data_ptr()), ctypes.c_void_p(grads.data_ptr()),
                ctypes.c_void_p(self.m1.data_ptr()), ctypes.c_void_p(self.m2.data_ptr()), self.step,
                ctypes.c_float(lr), ctypes.c_float(0.9), ctypes.c_float(0.999), ctypes.c_float(1e-8), st,
            ),
            "ndrr_proposal_adam",
        )
        return loss

    def gradients(self, X, T, V, alpha: float = 20.0) -> tuple[torch.Tensor, torch.Tensor]:
        """(grads [8450], loss) of the mean loss over the batch, no update."""
        lib = _ffi.load()
        grads = torch.zeros_like(self.params)
        loss = torch.zeros(1, device=self.device)
        n = X.shape[0]
        _prop_check(
            lib.ndrr_proposal_train_step(
                ctypes.c_void_p(self.params.data_ptr()), ctypes.c_void_p(X.data_ptr()),
                ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(V.data_ptr()), ctypes.c_int64(n),
                ctypes.c_float(alpha), ctypes.c_float(1.0 / max(1, n)), ctypes.c_void_p(grads.data_ptr()),
                ctypes.c_void_p(loss.data_ptr()), ctypes.c_void_p(_stream(self.device)),
            ),
            "ndrr_proposal_train_step",
        )
        return grads, loss

    def forward(self, X) -> torch.Tensor:
        """fp32 network outputs [R, 2] (the training-precision network)."""
        out = torch.empty(X.shape[0], 2, device=self.device)
        _prop_check(
            _ffi.load().ndrr_proposal_forward(
                ctypes.c_void_p(self.params.data_ptr()), ctypes.c_void_p(X.data_ptr()), ctypes.c_int64(X.shape[0]),
                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(_stream(self.device)),
            ),
            "ndrr_proposal_forward",
        )
        return out

    def pack(self) -> torch.Tensor:
        _prop_check(
            _ffi.load().ndrr_proposal_pack(
                ctypes.c_void_p(self.params.data_ptr()), ctypes.c_void_p(self.packed.data_ptr()),
                ctypes.c_void_p(_stream(self.device)),
            ),
            "ndrr_proposal_pack",
        )
        return self.packed

    def fit(self, X, T, V, epochs: int = 30, batch: int = 65536, lr: float = 2e-3, alpha: float = 20.0,
            seed: int = 0) -> list[float]:
        """Minibatch Adam over the dataset; returns the mean loss per epoch."""
        n = X.shape[0]
        g = torch.Generator(device=self.device).manual_seed(seed)
        history = []
        for ep in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=g)
            lr_ep = lr * (0.5 * (1 + math.cos(math.pi * ep / max(1, epochs))))  # cosine decay
            tot = torch.zeros(1, device=self.device)
            nb = 0
            for i in range(0, n, batch):
                idx = perm[i : i + batch]
                tot += self.train_step(X[idx].contiguous(), T[idx].contiguous(), V[idx].contiguous(), alpha, lr_ep)
                nb += 1
            history.append(float(tot) / max(1, nb))
        self.pack()
        return history

    def state_dict(self) -> dict:
        return {"params": self.params.detach().cpu(), "step": self.step}

    def load_state_dict(self, d: dict) -> None:
        self.params.copy_(d["params"].to(self.device))
        self.step = int(d.get("step", 0))
        self.pack()


@dataclass
class EmptySpace:
    """Skip configuration attached to a subject (`subject.empty_space`)."""

    grid: OccupancyGrid
    mode: int = _ffi.NDRR_SKIP_OCCUPANCY
    network: ProposalNetwork | None = None
    margin: float = 2.0  # samples of widening around a proposed interval
    # True: the occupancy skip runs inside the render kernels; False: per-ray
    # windows are computed first by their own kernel (ndrr_skip_windows) and
    # shared by the forward and the pose/camera adjoint of a step. Same
    # samples either way. The learned proposal always takes the window route.
    fused: bool = True

    @property
    def packed(self) -> torch.Tensor:
        if self.network is None:
            return torch.empty(0, dtype=torch.uint8, device=self.grid.grid.device)
        return self.network.packed

    @classmethod
    def occupancy(cls, vol: torch.Tensor, cell: int = 4, max_dist: int = 16, fused: bool = True) -> "EmptySpace":
        return cls(OccupancyGrid.build(vol, cell, max_dist), _ffi.NDRR_SKIP_OCCUPANCY, fused=fused)

    @classmethod
    def proposal(cls, vol: torch.Tensor, network: ProposalNetwork, cell: int = 4, max_dist: int = 16,
                 margin: float = 2.0) -> "EmptySpace":
        """Learned proposal checked by the occupancy grid, evaluated by the
        window kernel ahead of the march (ndrr_skip_windows)."""
        return cls(OccupancyGrid.build(vol, cell, max_dist), _ffi.NDRR_SKIP_PROPOSAL, network, margin, False)


def extents(vol, M, src, tgt, step, n_samples, width) -> torch.Tensor:
    """Per-ray non-empty interval [B, N, 2] (in t) from the plain forward."""
    B, N, _ = tgt.shape
    ext = torch.empty(B, N, 2, device=vol.device)
    raymarch_forward(vol, vol, M, src, tgt, step, n_samples, 1, width, extent=ext)
    return ext


def train_proposal(vol, M, src, tgt, step, n_samples, width, epochs=30, batch=65536, lr=2e-3, alpha=20.0,
                   seed=0, network: ProposalNetwork | None = None, cell: int = 4, widen_voxels: float | None = None):
    """Label the rays of the given poses with the plain renderer and fit the
    proposal network on them. Targets are widened beyond the occupancy
    check's resolution (grid cells of `cell` voxels, dilated by 2) so that a
    slightly-off prediction still passes the check: `cell + 12` voxels by
    default, which on the benchmark phantom gave the fewest fallbacks for the
    samples added (4 % of rays fall back at cell 4, against 19 % at cell + 3).
    Returns (network, losses)."""
    ext = extents(vol, M, src, tgt, step, n_samples, width)
    widen = float(cell + 12) if widen_voxels is None else float(widen_voxels)
    X, T, V = ProposalNetwork.dataset(vol, M, src, tgt, n_samples, width, ext, widen_voxels=widen)
    net = network or ProposalNetwork(vol.device, seed)
    hist = net.fit(X, T, V, epochs, batch, lr, alpha, seed)
    return net, hist
