"""Shared helpers of the test suite: build the same scene for the product and for the oracle."""
from __future__ import annotations

from pathlib import Path
from typing import List, Optional, Sequence

import numpy as np

from deepdrr_gb300 import geo, tables
from deepdrr_gb300.volume import Volume
from oracle import oracle

ROOT = Path(__file__).resolve().parent.parent
GOLDEN_TABLES = ROOT / "tests" / "golden" / "tables.npz"


def material_list(volumes: Sequence[Volume], attenuate: bool = False) -> List[str]:
    mats = []
    for v in volumes:
        mats.extend(v.materials[0].keys())
    if attenuate:
        mats.append("air")
    return sorted(set(mats))


def labels_for(volume: Volume, all_materials: Sequence[str]) -> np.ndarray:
    """Label remap of projector.py:1495-1519: volume material id -> index in the sorted list."""
    names, seg = volume.materials
    lut = np.zeros(max(names.values()) + 1, dtype=np.uint8)
    for name, idx in names.items():
        lut[idx] = all_materials.index(name)
    return lut[seg]


def oracle_scene(volumes: Sequence[Volume], proj, *, step: float = 0.1, spectrum="90KV_AL40",
                 priorities: Optional[Sequence[int]] = None, attenuate: bool = False,
                 max_ray_length: float = -4.0, frac_bits: int = 8, source=None,
                 density_dtype: str = "float32") -> oracle.Scene:
    """The oracle's scene for ``volumes`` seen from ``proj``. With a float16 / bfloat16
    ``density_dtype`` the densities are rounded to that type and the filtered samples to float16,
    which is what the projector's half-precision textures hold and return."""
    src = source or tables.NpzTables(GOLDEN_TABLES)
    mats = material_list(volumes, attenuate)
    e, pdf, mu = tables.build_tables(spectrum, mats, src)
    W, s, w, h = geo.view_arrays(proj)
    vols = [dict(density=quantize_density(v.data, density_dtype), labels=labels_for(v, mats),
                 ijk_from_world=v.ijk_from_world.data) for v in volumes]
    return oracle.Scene(vols, W, s, width=w, height=h, step=step, energies=e, pdf=pdf, mu=mu,
                        priorities=priorities, enabled=[1 if v.enabled else 0 for v in volumes],
                        max_ray_length=max_ray_length, attenuate_outside=attenuate,
                        air_index=mats.index("air") if attenuate else 0, frac_bits=frac_bits,
                        half_filter=density_dtype != "float32")


def scene_from_record(rec, name: str, world_from_index, source_world, width: int, height: int) -> oracle.Scene:
    """The oracle's scene for one view of a scene recorded in ``tests/golden/ref_kernel.npz``: volumes
    named by ``{name}__volumes`` (``{key}__density`` / ``__labels`` / ``__ijk_from_world``), tables
    and ``{name}__params`` = (step, max_ray_length, attenuate, air_index)."""
    vols = [dict(density=rec[f"{k}__density"], labels=rec[f"{k}__labels"], ijk_from_world=rec[f"{k}__ijk_from_world"])
            for k in (str(x) for x in rec[f"{name}__volumes"])]
    step, max_ray_length, attenuate, air_index = (float(x) for x in rec[f"{name}__params"])
    return oracle.Scene(vols, world_from_index, source_world, width=int(width), height=int(height), step=step,
                        energies=rec[f"{name}__energies"], pdf=rec[f"{name}__pdf"], mu=rec[f"{name}__mu"],
                        priorities=[int(p) for p in rec[f"{name}__priorities"]],
                        enabled=[int(e) for e in rec[f"{name}__enabled"]], max_ray_length=max_ray_length,
                        attenuate_outside=bool(attenuate), air_index=int(air_index))


def quantize_density(data: np.ndarray, density_dtype: str) -> np.ndarray:
    """Densities as stored: float32 unchanged, float16 / bfloat16 rounded to nearest even."""
    if density_dtype == "float32":
        return data
    if density_dtype == "float16":
        return data.astype(np.float16).astype(np.float32)
    import torch

    return torch.from_numpy(np.ascontiguousarray(data, dtype=np.float32)).bfloat16().float().numpy()


def uniform_cube(n: int = 32, density: float = 1.0, spacing: float = 1.0, material: str = "soft tissue") -> Volume:
    data = np.full((n, n, n), density, dtype=np.float32)
    origin = -(n - 1) / 2 * spacing * np.ones(3)
    return Volume.from_parameters(data, {material: np.ones((n, n, n), dtype=bool)}, origin=origin,
                                  spacing=(spacing,) * 3)


def axis_view(direction, sensor=(16, 16), pixel=0.5, sdd=1000.0, fraction=0.5, point=(0.0, 0.0, 0.0),
              up=(0.0, 0.0, 1.0)):
    return geo.CameraProjection.from_view(point, direction, up, source_to_detector_distance=sdd, pixel_size=pixel,
                                          sensor_size=sensor, source_to_point_fraction=fraction)


def rel_err(a, b, floor: float = 0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


class DeltaTables(tables.TableSource):
    """One 1 keV bin with pdf 1 and mu/rho = 1 for material `name`, 0 otherwise: then
    photon_prob = exp(-area_density[name]), which exposes the reference kernel's path lengths."""

    SPECTRUM = np.array([[1000.0, 1.0]])

    def __init__(self, name):
        self.name = name

    def spectrum(self, name):
        return self.SPECTRUM

    def has_material(self, material):
        return True

    def mu_over_rho(self, material, energies_kev, spectrum_name=None):
        return np.full(np.shape(energies_kev), 1.0 if material == self.name else 0.0, dtype=np.float32)
