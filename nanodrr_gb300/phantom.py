"""Seeded synthetic CT phantoms and pose sets for tests and benchmarks.

The recipe (one body ellipsoid of soft tissue in air with six bone ellipsoids,
HU converted by μ = 0.02 (1 + HU/1000) 1/mm) is defined on a 128 mm cube with
body semi-axes 60/45/60 mm and bone semi-axes 5-15 mm, and is scaled per axis
to any other extent. Labels: 0 air (HU threshold -500), 1 soft tissue,
2..7 the six bone ellipsoids (membership). Everything is generated from one
seed with a CPU generator, so a phantom is identical on every machine.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from .geometry import make_k_inv, make_rt_inv
from .subject import Subject

_REF_EXTENT = 128.0  # mm, the extent the recipe's sizes are quoted for


@dataclass
class Phantom:
    hu: torch.Tensor        # [D, H, W] float32
    mu: torch.Tensor        # [D, H, W] float32 (1/mm)
    label: torch.Tensor     # [D, H, W] uint8, classes 0..7
    spacing: tuple          # (sx, sy, sz) mm

    def subject(self, dtype=torch.float32, with_labels: bool = False, device=None) -> Subject:
        """Subject holding μ directly (convert_to_mu=False), centred at 0."""
        vol = self.mu.to(device=device, dtype=dtype)
        lab = self.label.to(device=device, dtype=torch.float32) if with_labels else None
        return Subject.from_volume(
            vol, self.spacing, label=lab, max_label=7 if with_labels else 0, convert_to_mu=False
        )


def make_phantom(shape=(128, 128, 128), spacing=(1.0, 1.0, 1.0), seed: int = 0, device="cpu",
                 body_scale: float = 1.0) -> Phantom:
    """Phantom of `shape` = (D, H, W) voxels with (sx, sy, sz) mm spacing.
    `body_scale` < 1 shrinks the body and bones relative to the extent (more
    air around them; 1 is the recipe)."""
    D, H, W = shape
    sx, sy, sz = spacing
    g = torch.Generator().manual_seed(seed)
    ext = torch.tensor([W * sx, H * sy, D * sz], dtype=torch.float64)
    scale = ext / _REF_EXTENT * float(body_scale)

    def u(lo, hi, n=None):
        r = torch.rand(() if n is None else (n,), generator=g, dtype=torch.float64)
        return lo + (hi - lo) * r

    body = torch.tensor([60.0, 45.0, 60.0], dtype=torch.float64) * scale
    bones = []
    for _ in range(6):
        axes = u(5.0, 15.0, 3) * scale
        # centre inside the body at up to 55 % of its semi-axes
        d = torch.randn(3, generator=g, dtype=torch.float64)
        d = d / d.norm() * u(0.0, 0.55)
        centre = d * body
        hu = u(400.0, 1500.0)
        ang = u(0.0, math.pi, 3)
        bones.append((centre, axes, hu, ang))
    # low-frequency tissue variation in [0, 80] HU
    waves = [(u(0.5, 2.0, 3), u(0.0, 2 * math.pi)) for _ in range(3)]
    noise = torch.randn(D, H, W, generator=g, dtype=torch.float32) * 10.0

    dev = torch.device(device)
    z = (torch.arange(D, device=dev, dtype=torch.float32) - (D - 1) / 2) * sz
    y = (torch.arange(H, device=dev, dtype=torch.float32) - (H - 1) / 2) * sy
    x = (torch.arange(W, device=dev, dtype=torch.float32) - (W - 1) / 2) * sx
    Z, Y, X = torch.meshgrid(z, y, x, indexing="ij")
    bx, by, bz = (float(v) for v in body)
    inside = (X / bx) ** 2 + (Y / by) ** 2 + (Z / bz) ** 2 <= 1.0
    field = torch.zeros_like(X)
    for k, ph in waves:
        kx, ky, kz = (float(v) for v in k)
        field += torch.sin(2 * math.pi * (kx * X / bx + ky * Y / by + kz * Z / bz) / 4 + float(ph))
    tissue = 40.0 + 40.0 * field / 3.0
    hu = torch.where(inside, tissue + noise.to(dev), torch.full_like(X, -1000.0))
    label = torch.where(hu > -500.0, 1, 0).to(torch.uint8)
    for i, (c, axes, bh, ang) in enumerate(bones):
        R = _rot(ang).to(dev)
        P = torch.stack([X - float(c[0]), Y - float(c[1]), Z - float(c[2])], dim=-1) @ R
        a = axes.float().to(dev)
        m = ((P / a) ** 2).sum(-1) <= 1.0
        m = m & inside
        hu = torch.where(m, torch.full_like(hu, float(bh)), hu)
        label = torch.where(m, torch.full_like(label, 2 + i), label)
    mu = (0.02 * (1.0 + hu / 1000.0)).clamp(min=0.0)
    return Phantom(hu=hu.contiguous(), mu=mu.contiguous(), label=label.contiguous(), spacing=(sx, sy, sz))


def _rot(ang: torch.Tensor) -> torch.Tensor:
    a, b, c = (float(v) for v in ang)
    Rz = torch.tensor([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])
    Rx = torch.tensor([[1, 0, 0], [0, math.cos(b), -math.sin(b)], [0, math.sin(b), math.cos(b)]])
    Ry = torch.tensor([[math.cos(c), 0, math.sin(c)], [0, 1, 0], [-math.sin(c), 0, math.cos(c)]])
    return (Rz @ Rx @ Ry).float()


def random_poses(n: int, seed: int = 1, rot_deg: float = 30.0, trans_mm: float = 50.0, sod: float = 600.0):
    """[n, 4, 4] camera-to-world poses: ZXY Euler angles uniform in
    ±rot_deg, camera centre (0, sod, 0) + uniform ±trans_mm per axis, AP."""
    g = torch.Generator().manual_seed(seed)
    rot = (torch.rand(n, 3, generator=g) * 2 - 1) * rot_deg
    trans = torch.tensor([0.0, sod, 0.0]) + (torch.rand(n, 3, generator=g) * 2 - 1) * trans_mm
    return make_rt_inv(rot, trans, orientation="AP", isocenter=torch.zeros(3))


def identity_pose(sod: float = 600.0):
    """Single AP pose with identity rotation, source `sod` mm from the isocenter."""
    return make_rt_inv(torch.zeros(1, 3), torch.tensor([[0.0, sod, 0.0]]), orientation="AP", isocenter=torch.zeros(3))


def detector(sdd: float = 1020.0, pixel: float = 1.4, height: int = 200, width: int = 200):
    """(k_inv [1, 3, 3], sdd [1]) of a centred detector."""
    return make_k_inv(sdd, pixel, pixel, 0.0, 0.0, height, width), torch.tensor([sdd])
