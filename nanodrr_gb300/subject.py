"""CT subject: the attenuation volume the renderer reads, its label map and
the voxel / world / grid affines.

Interface of the reference's `Subject` (nanodrr src/nanodrr/data/subject.py:
43-137): constructor arguments, the `image` property (HU -> μ on demand,
preprocess.py:9-50), the assignable `_image_hu` buffer its tests swap for a
leaf that requires a gradient (tests/drr/test_fused.py:116), the conversion
settings `convert_to_mu`, `mu_water`, `mu_bone`, `hu_bone` and `set_mu`,
`label`, `n_classes`, and the affines `world_to_voxel`, `voxel_to_world`,
`voxel_to_grid`, `world_to_grid`, `isocenter` (subject.py:81-88, 218-242).
File loading through torchio (subject.py:139-209) is replaced by
`Subject.from_volume`, which takes arrays already in memory.

How the μ volume is kept: every change of a conversion setting bumps a
revision number, and the converted volume is stored with the revision and
the identity (weak reference) and version counter of the HU tensor it came
from. `image` returns it while all three still match and converts again
otherwise, so a new setting, a new HU tensor (assigned, moved by `.to()`,
cast by `.double()`) or an in-place edit of the HU values is never served a
stale volume. On CUDA the conversion is one kernel of this library
(`ndrr_hu_to_mu`); when the conversion itself must be differentiable (the HU
tensor requires a gradient, or a setting is a tensor) it is the torch
expression of the same formula.
"""

from __future__ import annotations

import ctypes
import weakref

import torch

# Linear attenuation of water and cortical bone (1/mm, ~70 keV) and the HU of
# cortical bone: the reference's defaults (preprocess.py:4-6).
MU_WATER = 0.0192
MU_BONE = 0.0573
HU_BONE = 1000.0

_SETTING_DEFAULTS = {"convert_to_mu": True, "mu_water": MU_WATER, "mu_bone": MU_BONE, "hu_bone": HU_BONE}


def _hu_to_mu_torch(hu: torch.Tensor, mu_water, mu_bone, hu_bone) -> torch.Tensor:
    # Below 0 HU: air-water line through (-1000, 0) and (0, mu_water); above:
    # water-bone line through (0, mu_water) and (hu_bone, mu_bone). HU is
    # clamped at -1000 first and μ at 0 last.
    h = torch.clamp(hu, min=-1000.0)
    below = (h / 1000.0 + 1.0) * mu_water
    above = mu_water + (h / hu_bone) * (mu_bone - mu_water)
    return torch.clamp(torch.where(h > 0, above, below), min=0.0)


def _plain_number(v) -> bool:
    return isinstance(v, (int, float)) and not isinstance(v, bool)


def hu_to_mu(data: torch.Tensor, mu_water=MU_WATER, mu_bone=MU_BONE, hu_bone=HU_BONE) -> torch.Tensor:
    """Hounsfield units -> linear attenuation coefficients (1/mm), the
    reference's piecewise-linear air-water / water-bone map
    (preprocess.py:9-50). Float32/16/bf16 CUDA tensors that need no gradient
    through the conversion go through the library's elementwise kernel; other
    inputs use the torch expression of the same formula."""
    fast = (
        data.is_cuda
        and data.dtype in (torch.float32, torch.float16, torch.bfloat16)
        and not (torch.is_grad_enabled() and data.requires_grad)
        and all(_plain_number(v) for v in (mu_water, mu_bone, hu_bone))
    )
    if not fast:
        return _hu_to_mu_torch(data, mu_water, mu_bone, hu_bone)
    from . import _ffi
    from .raymarch import ndrr_dtype

    src = data.detach().contiguous()
    out = torch.empty_like(src)
    if src.numel():
        lib = _ffi.load()
        stream = torch.cuda.current_stream(src.device).cuda_stream
        _ffi.check(
            lib.ndrr_hu_to_mu(ctypes.c_void_p(src.data_ptr()), ndrr_dtype(src), ctypes.c_int64(src.numel()),
                              ctypes.c_float(mu_water), ctypes.c_float(mu_bone), ctypes.c_float(hu_bone),
                              ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream)),
            "ndrr_hu_to_mu",
        )
    return out


def _conversion_setting(name: str) -> property:
    """A HU -> μ conversion setting; assigning it bumps the revision, which
    makes the next `image` convert again."""

    def get(self):
        return self._mu_settings[name]

    def set_(self, value):
        self._mu_settings[name] = value
        self._mu_revision += 1

    return property(get, set_, doc=f"HU -> μ setting `{name}` (default {_SETTING_DEFAULTS[name]!r}).")


class Subject(torch.nn.Module):
    """Volume in [1, 1, D, H, W] with voxel (x, y, z) = element [z, y, x].

    Buffers (moved by `.to()` and saved in the state dict): `_image_hu`,
    `label`, `voxel_to_world`, `world_to_voxel`, `voxel_to_grid`,
    `world_to_grid` (= voxel_to_grid @ world_to_voxel) and `isocenter`.
    `**mu` takes the conversion settings `convert_to_mu`, `mu_water`,
    `mu_bone`, `hu_bone`; any other keyword raises TypeError."""

    convert_to_mu = _conversion_setting("convert_to_mu")
    mu_water = _conversion_setting("mu_water")
    mu_bone = _conversion_setting("mu_bone")
    hu_bone = _conversion_setting("hu_bone")

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
        unknown = [k for k in mu if k not in _SETTING_DEFAULTS]
        if unknown:
            raise TypeError(f"Unknown mu param(s): {', '.join(repr(k) for k in unknown)}")
        super().__init__()
        self._mu_settings = {**_SETTING_DEFAULTS, **mu}
        self._mu_revision = 0
        self._mu_state = None  # (revision, weakref to the HU tensor, its version, μ)
        tensors = {
            "_image_hu": imagedata,
            "label": labeldata,
            "voxel_to_world": voxel_to_world,
            "world_to_voxel": world_to_voxel,
            "voxel_to_grid": voxel_to_grid,
            "world_to_grid": voxel_to_grid @ world_to_voxel,
            "isocenter": isocenter,
        }
        for name, t in tensors.items():
            self.register_buffer(name, t)
        top = max_label if max_label is not None else int(labeldata.max().item())
        self.n_classes = int(top) + 1

    # --------------------------------------------------------------- μ volume
    def _mu_valid_for(self, hu: torch.Tensor) -> bool:
        st = self._mu_state
        return st is not None and st[0] == self._mu_revision and st[1]() is hu and st[2] == hu._version

    def _store_mu(self, hu: torch.Tensor, mu: torch.Tensor) -> torch.Tensor:
        self._mu_state = (self._mu_revision, weakref.ref(hu), hu._version, mu)
        return mu

    @property
    def image(self) -> torch.Tensor:
        """Attenuation volume [1, 1, D, H, W] (the HU values themselves when
        `convert_to_mu` is False), converted on first use and reused until a
        setting or the HU tensor changes."""
        hu = self._image_hu
        s = self._mu_settings
        if not s["convert_to_mu"]:
            return hu
        if self._mu_valid_for(hu):
            return self._mu_state[3]
        return self._store_mu(hu, hu_to_mu(hu, s["mu_water"], s["mu_bone"], s["hu_bone"]))

    def set_mu(self, mu_water=None, mu_bone=None, hu_bone=None) -> None:
        """Convert now with the given settings (floats or tensors, e.g. to
        differentiate through them) without changing the stored ones; the
        result is what `image` returns until a setting or the HU tensor
        changes. Omitted arguments use the stored settings."""
        s = self._mu_settings
        hu = self._image_hu
        chosen = [s[k] if v is None else v for k, v in (("mu_water", mu_water), ("mu_bone", mu_bone),
                                                         ("hu_bone", hu_bone))]
        self._store_mu(hu, hu_to_mu(hu, *chosen))

    # ------------------------------------------------------------ construction
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
        step = torch.tensor([float(s) for s in spacing], dtype=torch.float64)
        extent = torch.tensor([W - 1, H - 1, D - 1], dtype=torch.float64)
        start = -0.5 * extent * step if origin is None else torch.tensor(origin, dtype=torch.float64)
        v2w = torch.eye(4, dtype=torch.float64)
        v2w[:3, :3] = torch.diag(step)
        v2w[:3, 3] = start
        centre = start + 0.5 * extent * step
        image = volume[None, None]
        lab = torch.zeros_like(image) if label is None else label[None, None]
        dev = volume.device
        return cls(
            image,
            lab,
            v2w.float().to(dev),
            torch.linalg.inv(v2w).float().to(dev),
            cls._make_voxel_to_grid(image.shape).to(dev),
            centre.float().to(dev),
            max_label,
            **mu,
        )

    @staticmethod
    def _make_voxel_to_grid(shape) -> torch.Tensor:
        """Voxel index -> grid_sample's normalised coordinate with
        align_corners=False, per axis (x: W, y: H, z: D): the voxel extent
        [-0.5, S - 0.5] maps onto [-1, 1], so i -> (2 i + 1) / S - 1."""
        *_, D, H, W = shape
        mat = torch.eye(4, dtype=torch.float32)
        for axis, size in enumerate((W, H, D)):
            mat[axis, axis] = 2.0 / size
            mat[axis, 3] = 1.0 / size - 1.0
        return mat
