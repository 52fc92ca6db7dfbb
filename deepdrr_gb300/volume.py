"""CT volumes as the projector consumes them: densities, a material label volume, a pose.

Restates the parts of deepdrr/vol/volume.py (deepdrr v1.2.2) that the projection path reads:

* ``Volume.__init__`` (volume.py:152-192): ``data`` is a float32 [i, j, k] density array in g/cm^3,
  ``materials`` is a dict of binary masks or a ``(name -> id, label array)`` tuple;
* ``_format_materials`` (volume.py:955-992): label = enumeration index of the mask, last mask wins;
* ``_convert_hounsfield_to_density`` (volume.py:339-351) and the thresholding of
  deepdrr/load_dicom.py:132-143 behind ``from_hu``;
* ``from_parameters`` / ``world_from_ijk`` / ``IJK_from_world`` / ``translate`` / ``rotate`` / ``enabled``
  (volume.py:214-302, renderable.py:59-72, 156-192).

File loaders (NIfTI, NRRD, DICOM), cropping and isosurfaces are not part of the projection path.
"""
from __future__ import annotations

from typing import Any, Dict, Optional, Tuple, Union

import numpy as np

from .geo import FrameTransform


def hu_to_density(hu_values: np.ndarray, smooth_air: bool = False) -> np.ndarray:
    """Piecewise-linear HU -> g/cm^3 (volume.py:339-351): max(min(0.001029 HU + 1.030,
    0.0005886 HU + 1.03), 0)."""
    hu = np.asarray(hu_values)
    if smooth_air:
        hu = hu.copy()
        hu[hu <= -900] = -1000
    return np.maximum(np.minimum(0.001029 * hu + 1.030, 0.0005886 * hu + 1.03), 0)


def segment_thresholds(hu_values: np.ndarray) -> Dict[str, np.ndarray]:
    """Threshold segmentation (load_dicom.py:132-143): air HU <= -800, soft tissue (-800, 350],
    bone > 350."""
    hu = np.asarray(hu_values)
    return {
        "air": hu <= -800,
        "soft tissue": (-800 < hu) & (hu <= 350),
        "bone": 350 < hu,
    }


def format_materials(materials: Dict[str, np.ndarray]) -> Tuple[Dict[str, int], np.ndarray]:
    """Masks -> (name -> id, uint16 labels): id = enumeration index, later masks overwrite earlier
    ones (volume.py:955-992)."""
    seg = None
    mat_dict: Dict[str, int] = {}
    for mat_id, name in enumerate(materials):
        mask = np.asarray(materials[name]) > 0
        if seg is None:
            seg = np.zeros(mask.shape, dtype=np.uint16)
        seg[mask] = mat_id
        mat_dict[name] = mat_id
    if seg is None:
        raise ValueError("materials must contain at least one mask")
    return mat_dict, seg


class Volume:
    """A density volume with its material labels and its pose in world coordinates."""

    def __init__(self, data: np.ndarray,
                 materials: Union[Dict[str, np.ndarray], Tuple[Dict[str, int], np.ndarray]],
                 anatomical_from_IJK: Optional[FrameTransform] = None,
                 world_from_anatomical: Optional[FrameTransform] = None,
                 anatomical_coordinate_system: Optional[str] = None,
                 cache_dir: Optional[str] = None,
                 config: Optional[Dict[str, Any]] = None,
                 enabled: bool = True,
                 **kwargs) -> None:
        data = np.asarray(data)
        if data.ndim != 3:
            raise AssertionError("Volume data must be 3D.")
        self.data = np.array(data, dtype=np.float32)
        if isinstance(materials, tuple):
            self.materials = (dict(materials[0]), np.asarray(materials[1]).astype(np.uint16))
        else:
            self.materials = format_materials(materials)
        if self.materials[1].shape != self.data.shape:
            raise ValueError(f"label volume {self.materials[1].shape} does not match data {self.data.shape}")
        self.anatomical_from_IJK = FrameTransform(anatomical_from_IJK) if anatomical_from_IJK is not None \
            else FrameTransform.identity()
        self.world_from_anatomical = FrameTransform(world_from_anatomical) if world_from_anatomical is not None \
            else FrameTransform.identity()
        if anatomical_coordinate_system not in ("LPS", "RAS", None):
            raise AssertionError("anatomical_coordinate_system must be 'LPS', 'RAS' or None")
        self.anatomical_coordinate_system = anatomical_coordinate_system
        self.cache_dir = cache_dir
        self.config = dict(config or {})
        self.enabled = bool(enabled)

    # ---- constructors -----------------------------------------------------------------------
    @classmethod
    def from_parameters(cls, data: np.ndarray, materials, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0),
                        anatomical_coordinate_system: Optional[str] = None,
                        world_from_anatomical: Optional[FrameTransform] = None, **kwargs) -> "Volume":
        """Axis-aligned voxels: ``anatomical_from_IJK = [diag(spacing) | origin]``."""
        a_from_ijk = FrameTransform.from_scaling(spacing, origin)
        return cls(data, materials, anatomical_from_IJK=a_from_ijk, world_from_anatomical=world_from_anatomical,
                   anatomical_coordinate_system=anatomical_coordinate_system, **kwargs)

    @classmethod
    def from_hu(cls, hu_values: np.ndarray, origin=(0.0, 0.0, 0.0), use_thresholding: bool = True,
                spacing=(1.0, 1.0, 1.0), anatomical_coordinate_system: Optional[str] = None,
                world_from_anatomical: Optional[FrameTransform] = None, device=None, **kwargs) -> "Volume":
        """HU -> density and threshold segmentation (volume.py:281-302).

        With ``device`` (a CUDA device, or ``hu_values`` given as a CUDA tensor) the conversion runs
        on the GPU (drr_ingest_hu, same results bit for bit); the volume keeps the device arrays in
        the projector's layout and ``Projector.initialize`` uses them instead of uploading ``data``
        again, as long as ``data`` and the label array are the arrays made here."""
        if not use_thresholding:
            raise NotImplementedError("network segmentation is outside the projection path")
        on_gpu = device is not None or type(hu_values).__module__.startswith("torch")
        if not on_gpu:
            data = hu_to_density(hu_values).astype(np.float32)
            materials = segment_thresholds(hu_values)
            return cls.from_parameters(data, materials, origin=origin, spacing=spacing,
                                       anatomical_coordinate_system=anatomical_coordinate_system,
                                       world_from_anatomical=world_from_anatomical, **kwargs)
        import torch

        from .ingest import hu_to_density_and_labels

        hu = hu_values if isinstance(hu_values, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(hu_values))
        hu = hu.to(torch.device(device) if device is not None else hu.device)
        density, labels = hu_to_density_and_labels(hu)
        data = density.permute(2, 1, 0).cpu().numpy()
        ids = labels.permute(2, 1, 0).cpu().numpy().astype(np.uint16)
        names = {"air": 0, "soft tissue": 1, "bone": 2}
        vol = cls.from_parameters(data, (names, ids), origin=origin, spacing=spacing,
                                  anatomical_coordinate_system=anatomical_coordinate_system,
                                  world_from_anatomical=world_from_anatomical, **kwargs)
        vol._device_arrays = dict(density=density, labels=labels, data=vol.data, ids=vol.materials[1])
        return vol

    def device_arrays(self, device):
        """(density [nk, nj, ni] float32, material ids [nk, nj, ni] uint8) on ``device`` if this volume
        was ingested on the GPU and its arrays are unchanged, else None."""
        d = getattr(self, "_device_arrays", None)
        if d is None or d["data"] is not self.data or d["ids"] is not self.materials[1]:
            return None
        if d["density"].device != device:
            return None
        return d["density"], d["labels"]

    # ---- pose --------------------------------------------------------------------------------
    @property
    def world_from_ijk(self) -> FrameTransform:
        return self.world_from_anatomical @ self.anatomical_from_IJK

    @property
    def ijk_from_world(self) -> FrameTransform:
        return self.world_from_ijk.inverse()

    # the reference spells these with capitals too (renderable.py:59-72)
    @property
    def world_from_IJK(self) -> FrameTransform:
        return self.world_from_ijk

    @property
    def IJK_from_world(self) -> FrameTransform:
        return self.ijk_from_world

    def translate(self, t) -> "Volume":
        """Move the volume by ``t`` in world coordinates (renderable.py:156-166)."""
        self.world_from_anatomical = FrameTransform.from_rt(translation=np.asarray(t, dtype=np.float64)) \
            @ self.world_from_anatomical
        return self

    def rotate(self, rotation, center=None) -> "Volume":
        """Rotate about ``center`` (world; default the volume centre) by a 3x3 matrix
        (renderable.py:168-192)."""
        R = np.asarray(rotation, dtype=np.float64)
        c = self.center_in_world if center is None else np.asarray(center, dtype=np.float64)
        rot = FrameTransform.from_rt(translation=c) @ FrameTransform.from_rt(R) @ \
            FrameTransform.from_rt(translation=-c)
        self.world_from_anatomical = rot @ self.world_from_anatomical
        return self

    def set_enabled(self, enabled: bool) -> None:
        self.enabled = bool(enabled)

    # ---- geometry helpers -------------------------------------------------------------------
    @property
    def shape(self) -> Tuple[int, int, int]:
        return tuple(int(x) for x in self.data.shape)

    @property
    def spacing(self) -> np.ndarray:
        return np.abs(self.anatomical_from_IJK.R).max(axis=0)

    @property
    def center_in_world(self) -> np.ndarray:
        c = (np.array(self.shape, dtype=np.float64) - 1) / 2
        return self.world_from_ijk @ c

    def get_bounding_box_in_world(self) -> Tuple[np.ndarray, np.ndarray]:
        """Corners of the world-space box around the cell-centred voxels (volume.py:924-945)."""
        x, y, z = np.array(self.shape, dtype=np.float64) - 0.5
        corners = np.array([[a, b, c] for a in (-0.5, x) for b in (-0.5, y) for c in (-0.5, z)])
        w = np.array([self.world_from_ijk @ p for p in corners])
        return w.min(0), w.max(0)

    def __repr__(self) -> str:
        return f"Volume(shape={self.shape}, materials={list(self.materials[0])}, enabled={self.enabled})"
