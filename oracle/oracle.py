"""ctypes front end of the C oracle in ``drr_oracle.c``.

TEST INFRASTRUCTURE ONLY: the tests and ``__graft_entry__.smoke()`` check the product against it,
and the CPU-baseline leg of ``bench.py`` times it. The product package never imports it.

The host-side preparation follows deepdrr/projector/projector.py:802-831: the camera's
``world_from_index`` (3x3) and every volume's ``IJK_from_world`` (3x4) are float64 matrices cast to
float32, and the source position in each volume's IJK frame is computed in float64 and then cast.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB_PATH = BUILD / "libdrr_oracle.so"
MAX_VOL = 8
MAX_MAT = 16
# Multiply-add grouping of the reference kernel as nvcc 13.0 compiles it for sm_103a (found by
# matching the reference kernel's path lengths on GB300; see fp_profile in drr_oracle.c):
#   pixel ray     fma(u, w0, v*w1) + w2            (1)
#   squared norm  fma(z, z, fma(x, x, y*y))         (1 << 2)
#   IJK direction fma(a2, z, fma(a0, x, a1*y))      (1 << 4)
#   position      fma(alpha, r, s) - 1              (0 << 6)
#   label weights seg = fma(xy, z, seg)             (1 << 7)
REFERENCE_FP_PROFILE = 1 | (1 << 2) | (1 << 4) | (1 << 7)


class _Volume(ctypes.Structure):
    _fields_ = [
        ("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
        ("density", ctypes.c_void_p), ("labels", ctypes.c_void_p),
        ("priority", ctypes.c_int), ("enabled", ctypes.c_int),
        ("ijk_from_world", ctypes.c_float * 12), ("source_ijk", ctypes.c_float * 3),
        ("ijk_from_world_d", ctypes.c_double * 12), ("source_ijk_d", ctypes.c_double * 3),
        ("half_filter", ctypes.c_int),
    ]


class _Scene(ctypes.Structure):
    _fields_ = [
        ("n_volumes", ctypes.c_int), ("n_materials", ctypes.c_int),
        ("vol", _Volume * MAX_VOL),
        ("world_from_index", ctypes.c_float * 9), ("world_from_index_d", ctypes.c_double * 9),
        ("max_ray_length", ctypes.c_float), ("step", ctypes.c_float),
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("n_bins", ctypes.c_int),
        ("energies", ctypes.c_void_p), ("pdf", ctypes.c_void_p), ("mu", ctypes.c_void_p),
        ("attenuate_outside", ctypes.c_int), ("air_index", ctypes.c_int),
        ("frac_bits", ctypes.c_int), ("fp_profile", ctypes.c_int),
    ]


def build(force: bool = False) -> Path:
    """Compile ``drr_oracle.c`` into ``oracle/_build/libdrr_oracle.so`` (gcc, OpenMP, no FP contraction)."""
    src = HERE / "drr_oracle.c"
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= src.stat().st_mtime:
        return LIB_PATH
    BUILD.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(suffix=".so", dir=BUILD)
    os.close(fd)
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           str(src), "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.orc_project.restype = ctypes.c_int
        _lib.orc_project.argtypes = [ctypes.POINTER(_Scene), ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        _lib.orc_tex_linear.restype = ctypes.c_double
        _lib.orc_tex_linear.argtypes = [ctypes.POINTER(_Scene), ctypes.c_int] + [ctypes.c_double] * 3
        _lib.orc_ray_samples_f32.restype = ctypes.c_int
        _lib.orc_ray_samples_f32.argtypes = [ctypes.POINTER(_Scene), ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_tex_point.restype = ctypes.c_int
        _lib.orc_tex_point.argtypes = [ctypes.POINTER(_Scene), ctypes.c_int] + [ctypes.c_double] * 3
    return _lib


def source_in_ijk(ijk_from_world: np.ndarray, source_world: Sequence[float]) -> np.ndarray:
    """float64 ``IJK_from_world @ source`` in a fixed summation order ((a0 s0 + a1 s1) + a2 s2) + a3."""
    A = np.asarray(ijk_from_world, dtype=np.float64)
    s = [float(x) for x in source_world]
    out = np.zeros(3, dtype=np.float64)
    for r in range(3):
        a = [float(x) for x in A[r, :4]]
        out[r] = ((a[0] * s[0] + a[1] * s[1]) + a[2] * s[2]) + a[3]
    return out


class Scene:
    """Volumes + spectrum tables + one view, held alive for the C side."""

    def __init__(self, volumes, world_from_index, source_world, *, width, height, step, energies, pdf, mu,
                 priorities=None, enabled=None, max_ray_length=-1.0, attenuate_outside=False, air_index=0,
                 frac_bits=8, fp_profile=None, half_filter=False):
        nv = len(volumes)
        if nv > MAX_VOL:
            raise ValueError(f"the oracle holds at most {MAX_VOL} volumes")
        mu = np.ascontiguousarray(mu, dtype=np.float32)
        n_bins, M = mu.shape
        if M > MAX_MAT:
            raise ValueError(f"the oracle holds at most {MAX_MAT} materials")
        self._keep = []
        sc = _Scene()
        sc.n_volumes = nv
        sc.n_materials = M
        if priorities is None:
            priorities = [nv - 1 - i for i in range(nv)]
        if enabled is None:
            enabled = [1] * nv
        for i, v in enumerate(volumes):
            dens = np.ascontiguousarray(np.asarray(v["density"], dtype=np.float32).transpose(2, 1, 0))
            labs = np.ascontiguousarray(np.asarray(v["labels"], dtype=np.uint8).transpose(2, 1, 0))
            self._keep += [dens, labs]
            A = np.asarray(v["ijk_from_world"], dtype=np.float64)
            if A.shape == (3, 4):
                A = np.vstack([A, [0, 0, 0, 1]])
            s_ijk = source_in_ijk(A, source_world)
            ni, nj, nk = np.asarray(v["density"]).shape
            cv = sc.vol[i]
            cv.ni, cv.nj, cv.nk = ni, nj, nk
            cv.density = dens.ctypes.data
            cv.labels = labs.ctypes.data
            cv.priority = int(priorities[i])
            cv.half_filter = int(bool(half_filter[i] if isinstance(half_filter, (list, tuple)) else half_filter))
            cv.enabled = int(bool(enabled[i]))
            a32 = A[:3, :4].astype(np.float32).ravel()
            for j in range(12):
                cv.ijk_from_world[j] = float(a32[j])
                cv.ijk_from_world_d[j] = float(A[:3, :4].ravel()[j])
            s32 = s_ijk.astype(np.float32)
            for j in range(3):
                cv.source_ijk[j] = float(s32[j])
                cv.source_ijk_d[j] = float(s_ijk[j])
        W = np.asarray(world_from_index, dtype=np.float64)[:3, :3]
        w32 = W.astype(np.float32).ravel()
        for j in range(9):
            sc.world_from_index[j] = float(w32[j])
            sc.world_from_index_d[j] = float(W.ravel()[j])
        sc.max_ray_length = float(max_ray_length)
        sc.step = float(step)
        sc.width, sc.height = int(width), int(height)
        e = np.ascontiguousarray(energies, dtype=np.float32)
        p = np.ascontiguousarray(pdf, dtype=np.float32)
        assert e.shape == (n_bins,) and p.shape == (n_bins,)
        self._keep += [e, p, mu]
        sc.n_bins = n_bins
        sc.energies, sc.pdf, sc.mu = e.ctypes.data, p.ctypes.data, mu.ctypes.data
        sc.attenuate_outside = int(bool(attenuate_outside))
        sc.air_index = int(air_index)
        sc.frac_bits = int(frac_bits)
        sc.fp_profile = REFERENCE_FP_PROFILE if fp_profile is None else int(fp_profile)
        self.sc = sc
        self.n_materials = M

    def project(self, mode: str = "f32", ray_ids: Optional[np.ndarray] = None, threads: int = 0):
        """Run the oracle. Returns dict(intensity, photon_prob, area_density, samples).

        With ``ray_ids`` None the images are [H, W] (and [M, H, W]); otherwise flat [n] / [M, n]."""
        m = 0 if mode == "f32" else 1
        dt = np.float32 if m == 0 else np.float64
        W, H, M = self.sc.width, self.sc.height, self.n_materials
        if ray_ids is None:
            n = W * H
            ids_ptr = None
        else:
            ids = np.ascontiguousarray(ray_ids, dtype=np.int64)
            n = ids.shape[0]
            ids_ptr = ids.ctypes.data
        inten = np.zeros(n, dtype=dt)
        prob = np.zeros(n, dtype=dt)
        ad = np.zeros(M * n, dtype=dt)
        samples = ctypes.c_double(0.0)
        rc = lib().orc_project(ctypes.byref(self.sc), m, ids_ptr, n, inten.ctypes.data, prob.ctypes.data,
                               ad.ctypes.data, ctypes.byref(samples), int(threads))
        if rc != 0:
            raise ValueError("oracle rejected the scene")
        if ray_ids is None:
            inten, prob, ad = inten.reshape(H, W), prob.reshape(H, W), ad.reshape(M, H, W)
        else:
            ad = ad.reshape(M, n)
        return dict(intensity=inten, photon_prob=prob, area_density=ad, samples=samples.value)

    def ray_samples(self, u: int, v: int, cap: int = 1 << 20):
        """The float32-mode samples of ray (u, v) of a one-volume scene: (alpha [n], p [n, 3], weight [n]),
        float32, p in the shifted IJK frame of the march."""
        alpha = np.empty(cap, dtype=np.float32)
        p = np.empty((cap, 3), dtype=np.float32)
        w = np.empty(cap, dtype=np.float32)
        n = lib().orc_ray_samples_f32(ctypes.byref(self.sc), int(u), int(v), alpha.ctypes.data, p.ctypes.data,
                                      w.ctypes.data, cap)
        if n < 0 or n > cap:
            raise ValueError("ray_samples needs a one-volume scene and room for every sample")
        return alpha[:n], p[:n], w[:n]

    def tex_linear(self, vol: int, x: float, y: float, z: float) -> float:
        return lib().orc_tex_linear(ctypes.byref(self.sc), vol, x, y, z)

    def tex_point(self, vol: int, x: float, y: float, z: float) -> int:
        return lib().orc_tex_point(ctypes.byref(self.sc), vol, x, y, z)


def solid_angle(world_from_index: np.ndarray, width: int, height: int) -> np.ndarray:
    """Solid angle (sr) of every detector pixel seen from the source, float64 [height, width].

    Restates calculate_solid_angle, deepdrr/projector/project_kernel.cu:14-133: the pixel's corners
    (u, v), (u+1, v), (u+1, v+1), (u, v+1) become source-to-corner rays r = W [u, v, 1]; the pixel
    is split into the triangles (c0, c1, c2) and (c0, c2, c3), and each triangle's solid angle is
    2 atan2(|a . (b x c)|, abc + (a.b) c + (a.c) b + (b.c) a), plus pi where that is negative."""
    W = np.asarray(world_from_index, dtype=np.float64)[:3, :3]
    v, u = np.meshgrid(np.arange(height, dtype=np.float64), np.arange(width, dtype=np.float64), indexing="ij")
    corners = []
    for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1)):
        cu, cv = u + du, v + dv
        corners.append(np.stack([W[r, 0] * cu + W[r, 1] * cv + W[r, 2] for r in range(3)], -1))
    c0, c1, c2, c3 = corners
    mag = [np.linalg.norm(c, axis=-1) for c in corners]
    cross = np.cross(c0, c2)
    dot = lambda a, b: np.sum(a * b, axis=-1)  # noqa: E731

    def tri(a, b, c, ma, mb, mc, numer):
        om = 2.0 * np.arctan2(np.abs(numer), ma * mb * mc + dot(a, b) * mc + dot(a, c) * mb + dot(b, c) * ma)
        return np.where(om < 0.0, om + np.pi, om)

    return (tri(c0, c1, c2, mag[0], mag[1], mag[2], dot(c1, cross))
            + tri(c0, c2, c3, mag[0], mag[2], mag[3], dot(c3, cross)))


def neglog(images: np.ndarray, epsilon: float = 0.01) -> np.ndarray:
    """deepdrr/utils/image_utils.py:18-58 restated in numpy (note: it ADDS the per-image minimum)."""
    image = np.array(images, dtype=np.float32)
    squeeze = image.ndim == 2
    if squeeze:
        image = image[np.newaxis]
    image += image.min(axis=(1, 2), keepdims=True) + epsilon
    image = -np.log(image)
    lo = image.min(axis=(1, 2), keepdims=True)
    hi = image.max(axis=(1, 2), keepdims=True)
    if np.any(hi == lo):
        image[:] = 0
    else:
        image = (image - lo) / (hi - lo)
    return image[0] if squeeze else image


def collected_energy(intensity: np.ndarray, solid_angle: np.ndarray, photon_count: float, pixel_size_x: float,
                     pixel_size_y: float) -> np.ndarray:
    """Collected energy per pixel (keV / mm^2) of one [H, W] view, restating
    deepdrr/projector/projector.py:833-853 with numpy's float32 semantics: the float32 product of
    intensity and solid angle, times the photon count, over the float32 mean solid angle (numpy's
    own float32 mean), over the pixel area (a Python float, applied to the float32 array)."""
    inten = np.asarray(intensity, dtype=np.float32)
    sa = np.asarray(solid_angle, dtype=np.float32)
    mean = np.float32(sa.mean())
    e = (inten * sa) * np.float32(photon_count)
    e = e / mean
    return e / np.float32(pixel_size_x * pixel_size_y)
