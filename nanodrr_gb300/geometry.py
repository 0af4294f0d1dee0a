"""Host-side pose and camera construction (tiny tensors, plain torch).

Restates the parts of the reference's camera/geometry layers that build the
render call's inputs:
  - `transform_point` (nanodrr src/nanodrr/geometry/transform.py:15-28);
  - `make_k_inv` (src/nanodrr/camera/intrinsics.py:5-68);
  - `make_rt_inv` with the AP/PA/None re-orientations
    (src/nanodrr/camera/extrinsics.py:7-57, 94-110);
  - `convert` for the "euler", "so3_log" and "se3_log" parameterisations
    (src/nanodrr/geometry/se3.py:28-69, 179-221).
The reference delegates rotation conversions to the `roma` library (1.5.6,
uv.lock); the conversions here are written from their definitions: intrinsic
Euler angles compose left to right (R = R_a(α) R_b(β) R_c(γ) for convention
"abc"), lower-case conventions are extrinsic (reverse order), and a rotation
vector maps to a matrix by the Rodrigues formula.
"""

from __future__ import annotations

import math

import torch


def mm_small(A: torch.Tensor, B: torch.Tensor) -> torch.Tensor:
    """A @ B for small (3x3, 4x4) matrices as one broadcast multiply and sum:
    an elementwise kernel instead of a library GEMM launch per product, and
    deterministic under torch's deterministic mode."""
    return (A[..., :, :, None] * B[..., None, :, :]).sum(dim=-2)


def mv_small(A: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """A @ v for small matrices and vectors (broadcast multiply and sum)."""
    return (A * v[..., None, :]).sum(dim=-1)


def _homo(v: torch.Tensor) -> torch.Tensor:
    return torch.cat([v, torch.ones_like(v[..., :1])], dim=-1)


def transform_point(xform: torch.Tensor, v: torch.Tensor) -> torch.Tensor:
    """Apply homogeneous transforms [B, ..., N+1, N+1] to points [B, ..., N]."""
    h = torch.einsum("b...ij,b...j->b...i", xform, _homo(v))
    return h[..., :-1] / h[..., -1:]


def make_k_inv(
    sdd: float,
    delx: float,
    dely: float,
    x0: float,
    y0: float,
    height: int,
    width: int,
    dtype: torch.dtype | None = None,
    device: torch.device | str | None = None,
) -> torch.Tensor:
    """Inverse intrinsic matrix [1, 3, 3] of a cone-beam projector with focal
    lengths sdd/delta and the principal point offset (x0, y0) mm from the
    detector centre."""
    fx, fy = sdd / delx, sdd / dely
    cx = x0 / delx + width / 2.0
    cy = y0 / dely + height / 2.0
    return torch.tensor(
        [[[1.0 / fx, 0.0, -cx / fx], [0.0, 1.0 / fy, -cy / fy], [0.0, 0.0, 1.0]]],
        dtype=dtype,
        device=device,
    )


def _axis_rotation(axis: str, angle: torch.Tensor) -> torch.Tensor:
    c, s = torch.cos(angle), torch.sin(angle)
    o, z = torch.ones_like(angle), torch.zeros_like(angle)
    if axis == "x":
        rows = [o, z, z, z, c, -s, z, s, c]
    elif axis == "y":
        rows = [c, z, s, z, o, z, -s, z, c]
    elif axis == "z":
        rows = [c, -s, z, s, c, z, z, z, o]
    else:
        raise ValueError(f"bad axis {axis!r}")
    return torch.stack(rows, dim=-1).reshape(*angle.shape, 3, 3)


def euler_to_rotmat(convention: str, angles: torch.Tensor) -> torch.Tensor:
    """Rotation matrices [*, 3, 3] from Euler angles [*, 3] in radians.

    Upper-case conventions are intrinsic (each rotation about the already
    rotated frame, R = R1 @ R2 @ R3); lower-case ones are extrinsic (about the
    fixed frame, R = R3 @ R2 @ R1)."""
    if len(convention) != 3 or not (convention.isupper() or convention.islower()):
        raise ValueError(f"bad Euler convention {convention!r}")
    mats = [_axis_rotation(ax.lower(), angles[..., i]) for i, ax in enumerate(convention)]
    if convention.isupper():
        return mm_small(mm_small(mats[0], mats[1]), mats[2])
    return mm_small(mm_small(mats[2], mats[1]), mats[0])


def hat(v: torch.Tensor) -> torch.Tensor:
    """Skew-symmetric matrices [*, 3, 3] of vectors [*, 3]."""
    x, y, z = v.unbind(-1)
    o = torch.zeros_like(x)
    return torch.stack([o, -z, y, z, o, -x, -y, x, o], dim=-1).reshape(*v.shape[:-1], 3, 3)


def rotvec_to_rotmat(v: torch.Tensor) -> torch.Tensor:
    """Rodrigues formula R = I + a [v]x + b [v]x^2 with a = sin(θ)/θ and
    b = (1 - cos θ)/θ², using their Taylor series near θ = 0 so the map and
    its gradient stay finite at the identity."""
    th2 = (v * v).sum(-1)
    small = th2 < 1e-8
    th2s = torch.where(small, torch.ones_like(th2), th2)
    th = th2s.sqrt()
    a = torch.where(small, 1.0 - th2 / 6.0, torch.sin(th) / th)
    b = torch.where(small, 0.5 - th2 / 24.0, (1.0 - torch.cos(th)) / th2s)
    K = hat(v)
    eye = torch.eye(3, dtype=v.dtype, device=v.device).expand_as(K)
    return eye + a[..., None, None] * K + b[..., None, None] * mm_small(K, K)


def se3_V(v: torch.Tensor, eps: float = 1e-4) -> torch.Tensor:
    """V = I + ((1 - cos θ)/θ²)[ω]x + ((θ - sin θ)/θ³)[ω]x² of the SE(3)
    exponential (reference src/nanodrr/geometry/se3.py:197-221)."""
    th2 = (v * v).sum(-1)
    th = th2.clamp(min=eps).sqrt()
    K = hat(v)
    eye = torch.eye(3, dtype=v.dtype, device=v.device).expand_as(K)
    a = ((1.0 - torch.cos(th)) / th2)[..., None, None]
    b = ((th - torch.sin(th)) / (th2 * th))[..., None, None]
    return eye + a * K + b * mm_small(K, K)


def make_se3(R: torch.Tensor, t: torch.Tensor) -> torch.Tensor:
    T = torch.zeros(*R.shape[:-2], 4, 4, dtype=R.dtype, device=R.device)
    T[..., :3, :3] = R
    T[..., :3, 3] = t
    T[..., 3, 3] = 1.0
    return T


def convert(
    rotation: torch.Tensor,
    translation: torch.Tensor,
    parameterization: str,
    convention: str | None = None,
    degrees: bool = True,
    isocenter: torch.Tensor | None = None,
) -> torch.Tensor:
    """Pose [*, 4, 4] from a rotation parameterisation and a camera centre:
    t = R @ translation (+ isocenter), as the reference's `convert`."""
    if parameterization == "se3_log":
        R = rotvec_to_rotmat(rotation)
        t = mv_small(se3_V(rotation), translation)
        return make_se3(R, t)
    if parameterization == "euler":
        if convention is None:
            raise ValueError("convention must be specified for Euler angles (e.g., 'XYZ', 'ZYX')")
        ang = rotation * (math.pi / 180.0) if degrees else rotation
        R = euler_to_rotmat(convention, ang)
    elif parameterization == "so3_log":
        R = rotvec_to_rotmat(rotation)
    else:
        raise ValueError(f"unsupported parameterization {parameterization!r}")
    t = mv_small(R, translation)
    if isocenter is not None:
        t = t + isocenter
    return make_se3(R, t)


_ORIENTATIONS = {
    "AP": [[-1, 0, 0, 0], [0, 0, -1, 0], [0, -1, 0, 0], [0, 0, 0, 1]],
    "PA": [[-1, 0, 0, 0], [0, 0, 1, 0], [0, -1, 0, 0], [0, 0, 0, 1]],
    None: [[-1, 0, 0, 0], [0, -1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]],
}


def orientation_matrix(orientation: str | None, device=None, dtype=None) -> torch.Tensor:
    if orientation not in _ORIENTATIONS:
        raise ValueError(f"Unknown orientation {orientation!r}. Expected one of: 'AP', 'PA', or None.")
    return torch.tensor(_ORIENTATIONS[orientation], device=device, dtype=dtype)


def make_rt_inv(
    rotation: torch.Tensor,
    translation: torch.Tensor,
    orientation: str | None = "AP",
    isocenter: torch.Tensor | None = None,
) -> torch.Tensor:
    """Camera-to-world matrices [B, 4, 4] from ZXY Euler angles in degrees and
    a camera position relative to the isocenter: pose @ reorientation."""
    iso = isocenter if isocenter is not None else torch.zeros(3, device=rotation.device, dtype=rotation.dtype)
    pose = convert(rotation, translation, "euler", convention="ZXY", isocenter=iso)
    return mm_small(pose, orientation_matrix(orientation, rotation.device, rotation.dtype))
