"""CT subject container: attenuation volume, optional label map and affines.

Mirrors the reference's `Subject` (nanodrr src/nanodrr/data/subject.py:43-242)
for everything the render call reads: the cached HU -> μ image
(`image`, subject.py:98-107; conversion preprocess.py:9-50), the label map,
`n_classes` (subject.py:93-96) and the affines `world_to_voxel`,
`voxel_to_grid`, `world_to_grid` (subject.py:81-88, 218-242). File loading
through torchio (subject.py:139-209) is replaced by `Subject.from_volume`,
which takes arrays already in memory.
"""

from __future__ import annotations

import torch

MU_WATER = 0.0192
MU_BONE = 0.0573
HU_BONE = 1000.0

_MU_FIELDS = frozenset({"convert_to_mu", "mu_water", "mu_bone", "hu_bone"})


def hu_to_mu(data: torch.Tensor, mu_water=MU_WATER, mu_bone=MU_BONE, hu_bone=HU_BONE) -> torch.Tensor:
    """Piecewise-linear HU -> linear attenuation (1/mm): air-water below 0 HU,
    water-bone above, clamped to HU >= -1000 and μ >= 0."""
    hu = data.clamp(min=-1000.0)
    low = mu_water * (1.0 + hu / 1000.0)
    high = mu_water + (hu / hu_bone) * (mu_bone - mu_water)
    return torch.where(hu <= 0, low, high).clamp(min=0.0)


class _CachedParam:
    """Scalar μ parameter whose change invalidates the cached μ image."""

    def __init__(self, default) -> None:
        self.default = default

    def __set_name__(self, owner, name) -> None:
        self.name = f"_{name}"

    def __get__(self, obj, objtype=None):
        if obj is None:
            return self
        return getattr(obj, self.name, self.default)

    def __set__(self, obj, value) -> None:
        if getattr(obj, self.name, self.default) != value:
            setattr(obj, self.name, value)
            if hasattr(obj, "_image_mu_cache"):
                obj._image_mu_cache = None


class Subject(torch.nn.Module):
    """Volume in [1, 1, D, H, W] with voxel (x, y, z) = element [z, y, x]."""

    convert_to_mu = _CachedParam(True)
    mu_water = _CachedParam(MU_WATER)
    mu_bone = _CachedParam(MU_BONE)
    hu_bone = _CachedParam(HU_BONE)

    def __init__(
        self,
        imagedata: torch.Tensor,
        labeldata: torch.Tensor,
        voxel_to_world: torch.Tensor,
        world_to_voxel: torch.Tensor,
        voxel_to_grid: torch.Tensor,
        isocenter: torch.Tensor,
        max_label: int | None = None,
        **mu,
    ) -> None:
        unknown = mu.keys() - _MU_FIELDS
        if unknown:
            raise TypeError(f"Unknown mu param(s): {', '.join(repr(k) for k in unknown)}")
        super().__init__()
        self.register_buffer("_image_hu", imagedata)
        self.register_buffer("_image_mu_cache", None, persistent=False)
        self.register_buffer("label", labeldata)
        self.register_buffer("world_to_grid", voxel_to_grid @ world_to_voxel)
        self.register_buffer("isocenter", isocenter)
        self.register_buffer("voxel_to_world", voxel_to_world)
        self.register_buffer("world_to_voxel", world_to_voxel)
        self.register_buffer("voxel_to_grid", voxel_to_grid)
        for k, v in mu.items():
            setattr(self, k, v)
        self.n_classes = int(max_label + 1) if max_label is not None else int(self.label.max().item()) + 1

    @property
    def image(self) -> torch.Tensor:
        """μ volume (or the raw values when convert_to_mu is False), cached."""
        if not self.convert_to_mu:
            return self._image_hu
        if self._image_mu_cache is None:
            self._image_mu_cache = hu_to_mu(self._image_hu, self.mu_water, self.mu_bone, self.hu_bone)
        return self._image_mu_cache

    def to(self, *args, **kwargs) -> "Subject":
        had_cache = self._image_mu_cache is not None
        result = super().to(*args, **kwargs)
        if had_cache:
            result._image_mu_cache = hu_to_mu(result._image_hu, result.mu_water, result.mu_bone, result.hu_bone)
        return result

    def set_mu(self, mu_water=None, mu_bone=None, hu_bone=None) -> None:
        self._image_mu_cache = hu_to_mu(
            self._image_hu,
            mu_water if mu_water is not None else self.mu_water,
            mu_bone if mu_bone is not None else self.mu_bone,
            hu_bone if hu_bone is not None else self.hu_bone,
        )

    @classmethod
    def from_volume(
        cls,
        volume: torch.Tensor,
        spacing=(1.0, 1.0, 1.0),
        label: torch.Tensor | None = None,
        origin=None,
        max_label: int | None = None,
        **mu,
    ) -> "Subject":
        """Subject from a [D, H, W] array with (sx, sy, sz) mm voxels.

        `origin` is the world position of voxel (0, 0, 0); by default the
        volume is centred on the world origin, which is also the isocenter."""
        if volume.dim() != 3:
            raise ValueError("volume must be [D, H, W]")
        D, H, W = volume.shape
        sx, sy, sz = (float(s) for s in spacing)
        if origin is None:
            origin = (-(W - 1) / 2 * sx, -(H - 1) / 2 * sy, -(D - 1) / 2 * sz)
        v2w = torch.eye(4, dtype=torch.float64)
        v2w[0, 0], v2w[1, 1], v2w[2, 2] = sx, sy, sz
        v2w[:3, 3] = torch.tensor(origin, dtype=torch.float64)
        w2v = torch.linalg.inv(v2w)
        image = volume[None, None]
        lab = label[None, None] if label is not None else torch.zeros_like(image)
        center = v2w @ torch.tensor([(W - 1) / 2, (H - 1) / 2, (D - 1) / 2, 1.0], dtype=torch.float64)
        return cls(
            image,
            lab,
            v2w.float().to(volume.device),
            w2v.float().to(volume.device),
            cls._make_voxel_to_grid(image.shape).to(volume.device),
            center[:3].float().to(volume.device),
            max_label,
            **mu,
        )

    @staticmethod
    def _make_voxel_to_grid(shape) -> torch.Tensor:
        """Affine from voxel indices to grid_sample's [-1, 1] coordinates with
        align_corners=False: i -> (2 i + 1) / S - 1 per axis (x: W, y: H, z: D)."""
        *_, D, H, W = shape
        size = torch.tensor([W, H, D], dtype=torch.float32)
        mat = torch.eye(4, dtype=torch.float32)
        mat[:3, :3] = torch.diag(2.0 / size)
        mat[:3, 3] = 1.0 / size - 1.0
        return mat
