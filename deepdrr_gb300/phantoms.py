"""Seeded synthetic CT phantoms and C-arm poses for the projector's workloads.

The reference's only test volume (a downloaded chest CT) is not available offline, so these
generators stand in for it with CT-like HU distributions. HU values go through the reference's
own conversion rules (``Volume.from_hu``: hu_to_density, threshold segmentation), and metal is
labelled "titanium" with density 4.5 g/cm^3 through an explicit mask, the way
deepdrr/vol/volume.py:1857-1876 (MetalVolume) segments metal.

Workloads (sizes as the benchmark configurations define them):
  * ``simple``   n^3 volume at 1 mm: air, a soft-tissue ellipsoid (40 +- 20 HU), 3 bone ellipsoids
                  (uniform 700-1500 HU); air / soft tissue / bone.
  * ``ct``       512 x 512 x 400 at 0.8 x 0.8 x 1.0 mm: body, lungs (-800 HU), spine and ribs
                  (uniform 1000-1800 HU) and a titanium cylinder; air / bone / soft tissue / titanium.
  * ``implant``  a titanium mask volume (labels air / titanium, density 4.5 x mask).
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Tuple

import numpy as np

from .geo import CameraProjection, FrameTransform, rotation_from_rotvec
from .volume import Volume, hu_to_density, segment_thresholds

TITANIUM_DENSITY = 4.5


def _box(center, radius, shape):
    lo = [max(0, int(np.floor(c - r))) for c, r in zip(center, radius)]
    hi = [min(s, int(np.ceil(c + r)) + 1) for c, r, s in zip(center, radius, shape)]
    return tuple(slice(a, b) for a, b in zip(lo, hi)), lo


def _ellipsoid_mask(shape, center, axes, rot: Optional[np.ndarray] = None):
    """Boolean mask of an ellipsoid (voxel units) restricted to its bounding box."""
    r = np.max(axes) if rot is not None else np.asarray(axes)
    radius = np.broadcast_to(r, (3,))
    sl, lo = _box(center, radius, shape)
    ii = np.arange(sl[0].start, sl[0].stop, dtype=np.float32)[:, None, None] - center[0]
    jj = np.arange(sl[1].start, sl[1].stop, dtype=np.float32)[None, :, None] - center[1]
    kk = np.arange(sl[2].start, sl[2].stop, dtype=np.float32)[None, None, :] - center[2]
    if rot is not None:
        R = np.asarray(rot, dtype=np.float32)
        x = R[0, 0] * ii + R[1, 0] * jj + R[2, 0] * kk
        y = R[0, 1] * ii + R[1, 1] * jj + R[2, 1] * kk
        z = R[0, 2] * ii + R[1, 2] * jj + R[2, 2] * kk
    else:
        x, y, z = ii, jj, kk
    m = (x / axes[0]) ** 2 + (y / axes[1]) ** 2 + (z / axes[2]) ** 2 <= 1.0
    return sl, m


def simple_phantom_hu(n: int = 128, seed: int = 0) -> np.ndarray:
    """n^3 HU volume: air, soft-tissue ellipsoid (40 +- 20 HU noise), 3 bone ellipsoids."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    hu = np.full(shape, -1000.0, dtype=np.float32)
    c = np.array(shape, dtype=np.float64) / 2 + rng.uniform(-0.05, 0.05, 3) * n
    axes = rng.uniform(0.30, 0.42, 3) * n
    sl, m = _ellipsoid_mask(shape, c, axes)
    noise = (40.0 + 20.0 * rng.standard_normal(m.shape, dtype=np.float32)).astype(np.float32)
    hu[sl] = np.where(m, noise, hu[sl])
    for _ in range(3):
        bc = c + rng.uniform(-0.18, 0.18, 3) * n
        ba = rng.uniform(0.04, 0.12, 3) * n
        rot = rotation_from_rotvec(rng.normal(size=3))
        sl, m = _ellipsoid_mask(shape, bc, ba, rot)
        val = rng.uniform(700.0, 1500.0, m.shape).astype(np.float32)
        hu[sl] = np.where(m, val, hu[sl])
    return hu


def ct_phantom(shape=(512, 512, 400), spacing=(0.8, 0.8, 1.0), seed: int = 0,
               titanium: bool = True) -> Tuple[np.ndarray, dict]:
    """CT-like HU volume plus a titanium mask. Returns (hu float32, extra masks dict)."""
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape)
    sp = np.asarray(spacing, dtype=np.float64)
    hu = np.full(shape, -1000.0, dtype=np.float32)
    ni, nj, nk = shape
    ctr = np.array([ni / 2, nj / 2, nk / 2])
    # body: an elliptic cylinder-like ellipsoid, soft tissue 40 +- 20 HU
    body_axes = np.array([0.44 * ni, 0.34 * nj, 0.62 * nk])
    sl, m = _ellipsoid_mask(shape, ctr, body_axes)
    tissue = (40.0 + 20.0 * rng.standard_normal(m.shape, dtype=np.float32)).astype(np.float32)
    hu[sl] = np.where(m, tissue, hu[sl])
    # lungs: two ellipsoids at -800 HU (+- 20 HU noise)
    for side in (-1, 1):
        lc = ctr + np.array([side * 0.19 * ni, -0.03 * nj, 0.05 * nk]) + rng.uniform(-3, 3, 3)
        la = np.array([0.15 * ni, 0.2 * nj, 0.32 * nk]) * rng.uniform(0.92, 1.05, 3)
        sl, m = _ellipsoid_mask(shape, lc, la)
        lung = (-800.0 + 20.0 * rng.standard_normal(m.shape, dtype=np.float32)).astype(np.float32)
        hu[sl] = np.where(m, lung, hu[sl])
    # spine: a column of vertebra-like ellipsoids posterior of centre
    n_vert = 12
    for v in range(n_vert):
        z = (v + 0.5) / n_vert * nk
        vc = np.array([ctr[0], ctr[1] + 0.24 * nj, z]) + rng.uniform(-1.5, 1.5, 3)
        va = np.array([0.055 * ni, 0.055 * nj, 0.4 * nk / n_vert])
        sl, m = _ellipsoid_mask(shape, vc, va)
        bone = rng.uniform(1000.0, 1800.0, m.shape).astype(np.float32)
        hu[sl] = np.where(m, bone, hu[sl])
    # ribs: thin elliptic rings (tubes) in planes of constant k
    ii = np.arange(ni, dtype=np.float32)[:, None] - ctr[0]
    jj = np.arange(nj, dtype=np.float32)[None, :] - ctr[1]
    for r in range(10):
        z0 = (r + 1) / 11 * nk * 0.9 + 0.05 * nk
        a, b = 0.38 * ni * rng.uniform(0.95, 1.02), 0.28 * nj * rng.uniform(0.95, 1.02)
        rr = np.sqrt((ii / a) ** 2 + (jj / b) ** 2)
        ring = np.abs(rr - 1.0) * min(a, b) < 0.012 * ni
        k0, k1 = max(0, int(z0 - 0.01 * nk)), min(nk, int(z0 + 0.01 * nk) + 1)
        for k in range(k0, k1):
            vals = rng.uniform(1000.0, 1800.0, ring.shape).astype(np.float32)
            hu[:, :, k] = np.where(ring, vals, hu[:, :, k])
    masks = {}
    if titanium:
        # a small titanium cylinder (a screw) through the anterior body
        tc = ctr + np.array([0.08 * ni, -0.12 * nj, 0.1 * nk])
        ta = np.array([0.012 * ni, 0.012 * nj, 0.06 * nk])
        rot = rotation_from_rotvec(np.array([0.3, 0.2, 0.0]))
        sl, m = _ellipsoid_mask(shape, tc, ta, rot)
        tmask = np.zeros(shape, dtype=bool)
        tmask[sl] = m
        masks["titanium"] = tmask
    return hu, masks


def volume_from_hu(hu: np.ndarray, spacing=(1.0, 1.0, 1.0), origin=None, masks: Optional[dict] = None) -> Volume:
    """``Volume.from_hu`` with optional metal masks appended (last mask wins)."""
    sp = np.asarray(spacing, dtype=np.float64)
    if origin is None:
        origin = -(np.asarray(hu.shape, dtype=np.float64) - 1) / 2 * sp
    data = hu_to_density(hu).astype(np.float32)
    materials = segment_thresholds(hu)
    for name, m in (masks or {}).items():
        data[m] = TITANIUM_DENSITY if name == "titanium" else data[m]
        materials = {k: (v & ~m) for k, v in materials.items()}
        materials[name] = m
    return Volume.from_parameters(data, materials, origin=origin, spacing=sp)


def implant_volume(shape=(96, 96, 64), spacing=(0.5, 0.5, 0.5), seed: int = 0) -> Volume:
    """Titanium implant mask volume: labels air / titanium, density 4.5 x mask."""
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape)
    c = np.array(shape) / 2 + rng.uniform(-2, 2, 3)
    axes = np.array([0.18 * shape[0], 0.18 * shape[1], 0.45 * shape[2]])
    sl, m = _ellipsoid_mask(shape, c, axes, rotation_from_rotvec(rng.normal(size=3) * 0.3))
    mask = np.zeros(shape, dtype=bool)
    mask[sl] = m
    data = (TITANIUM_DENSITY * mask).astype(np.float32)
    sp = np.asarray(spacing, dtype=np.float64)
    origin = -(np.asarray(shape, dtype=np.float64) - 1) / 2 * sp
    return Volume.from_parameters(data, {"air": ~mask, "titanium": mask}, origin=origin, spacing=sp)


def random_rigid(rng, max_translation_mm: float, max_angle_deg: float) -> FrameTransform:
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    ang = np.deg2rad(rng.uniform(-max_angle_deg, max_angle_deg))
    t = rng.uniform(-1, 1, 3) * max_translation_mm
    return FrameTransform.from_rt(rotation_from_rotvec(axis * ang), t)


def random_views(n: int, center, seed: int = 0, *, sphere_mm: float = 100.0, cone_deg: float = 30.0,
                 axis=(0.0, 1.0, 0.0), up=(0.0, 0.0, 1.0), source_to_detector_distance: float = 1020.0,
                 pixel_size: float = 0.194, sensor_size=(1536, 1536),
                 fraction_range=(0.5, 0.9)) -> List[CameraProjection]:
    """Seeded C-arm views: target point uniform in a ``sphere_mm`` ball around ``center``, viewing
    direction uniform in a ``cone_deg`` cone around ``axis``, source-to-point fraction uniform in
    ``fraction_range`` of the source-to-detector distance."""
    rng = np.random.default_rng(seed)
    axis = np.asarray(axis, dtype=np.float64) / np.linalg.norm(axis)
    out = []
    for _ in range(n):
        while True:
            p = rng.uniform(-1, 1, 3)
            if np.dot(p, p) <= 1:
                break
        point = np.asarray(center, dtype=np.float64) + p * sphere_mm
        cos_max = np.cos(np.deg2rad(cone_deg))
        ct = rng.uniform(cos_max, 1.0)
        phi = rng.uniform(0, 2 * np.pi)
        st = np.sqrt(1 - ct * ct)
        a = np.array([1.0, 0.0, 0.0]) if abs(axis[0]) < 0.9 else np.array([0.0, 0.0, 1.0])
        e1 = np.cross(axis, a)
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(axis, e1)
        d = ct * axis + st * (np.cos(phi) * e1 + np.sin(phi) * e2)
        frac = rng.uniform(*fraction_range)
        out.append(CameraProjection.from_view(point, d, up, source_to_detector_distance=source_to_detector_distance,
                                              pixel_size=pixel_size, sensor_size=sensor_size,
                                              source_to_point_fraction=frac))
    return out


# ---- the benchmark workloads -------------------------------------------------------------------

def workload_simple(seed: int = 0, n: int = 128, views: int = 1, sensor=(256, 256), pixel=1.2):
    """128^3 phantom, 256^2 detector at 1.2 mm, SDD 1020, 120 kVp (M = 3)."""
    vol = volume_from_hu(simple_phantom_hu(n, seed), spacing=(1.0, 1.0, 1.0))
    projs = random_views(views, vol.center_in_world, seed=seed + 1, sphere_mm=0.0, cone_deg=30.0,
                         source_to_detector_distance=1020.0, pixel_size=pixel, sensor_size=sensor,
                         fraction_range=(0.5, 0.5))
    return [vol], projs, dict(step=0.1, spectrum="120KV_AL43", neglog=True)


def workload_ct(seed: int = 0, views: int = 32, shape=(512, 512, 400), sensor=(1536, 1536), pixel=0.194,
                spectrum: str = "90KV_AL40"):
    """512 x 512 x 400 CT phantom with titanium, 1536^2 detector at 0.194 mm, 32 poses, 90 kVp (M = 4)."""
    hu, masks = ct_phantom(shape, (0.8, 0.8, 1.0), seed)
    vol = volume_from_hu(hu, spacing=(0.8, 0.8, 1.0), masks=masks)
    projs = random_views(views, vol.center_in_world, seed=seed + 1, sphere_mm=100.0, cone_deg=30.0,
                         source_to_detector_distance=1020.0, pixel_size=pixel, sensor_size=sensor,
                         fraction_range=(0.5, 0.9))
    return [vol], projs, dict(step=0.1, spectrum=spectrum, neglog=True)


def workload_multi(seed: int = 0, views: int = 256, sensor=(384, 384), pixel: float = 0.3,
                   ct_shape=(512, 512, 400)):
    """Three overlapping volumes of uneven size, each with its own seeded rigid pose: the CT phantom
    (512 x 512 x 400), a 256^3 phantom at 1 mm and a 96 x 96 x 64 titanium implant mask; `views`
    seeded poses on a 384^2 detector at 0.3 mm, 90 kVp (M = 4)."""
    rng = np.random.default_rng(seed + 100)
    hu, masks = ct_phantom(ct_shape, (0.8, 0.8, 1.0), seed)
    ct = volume_from_hu(hu, spacing=(0.8, 0.8, 1.0), masks=masks)
    ph = volume_from_hu(simple_phantom_hu(256, seed=seed + 1), spacing=(1.0, 1.0, 1.0))
    ph.world_from_anatomical = random_rigid(rng, 40.0, 20.0)
    imp = implant_volume((96, 96, 64), seed=seed + 2)
    imp.world_from_anatomical = random_rigid(rng, 30.0, 45.0)
    projs = random_views(views, ct.center_in_world, seed=seed + 3, sphere_mm=100.0, cone_deg=30.0,
                         source_to_detector_distance=1020.0, pixel_size=pixel, sensor_size=sensor,
                         fraction_range=(0.5, 0.9))
    return [ct, ph, imp], projs, dict(step=0.1, spectrum="90KV_AL40", neglog=True)


def workload_adjoint(seed: int = 0, views: int = 64, n: int = 256, sensor=(256, 256), pixel: float = 2.0):
    """2D/3D registration case: the n^3 phantom at 1 mm (M = 3), `views` seeded poses on a 256^2
    detector at 2 mm (magnification 2), 90 kVp, and a target pose (t in mm, rotation vector in
    rad) perturbed by up to 5 mm and 5 degrees per axis."""
    rng = np.random.default_rng(seed + 200)
    vol = volume_from_hu(simple_phantom_hu(n, seed=seed), spacing=(1.0, 1.0, 1.0))
    projs = random_views(views, vol.center_in_world, seed=seed + 4, sphere_mm=5.0, cone_deg=60.0,
                         source_to_detector_distance=1020.0, pixel_size=pixel, sensor_size=sensor,
                         fraction_range=(0.5, 0.5))
    target = np.concatenate([rng.uniform(-5.0, 5.0, 3), np.deg2rad(rng.uniform(-5.0, 5.0, 3))])
    return [vol], projs, dict(step=0.1, spectrum="90KV_AL40", neglog=False, target_pose=target)
