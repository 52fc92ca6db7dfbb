"""Python front end of ``ref_harness.cu``: runs the reference's own projectKernel on the GPU.

TEST INFRASTRUCTURE ONLY (see ref_harness.cu). The cubins come from ``build_ref.build_cubins``;
when they are absent (no reference sources where the tree was built) ``available`` is False and
the tests that need them skip.
"""
from __future__ import annotations

import ctypes
from pathlib import Path
from typing import Optional

import numpy as np

from . import build_ref
from .oracle import Scene

_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(str(build_ref.build_harness()))
        _LIB.ref_last_error.restype = ctypes.c_char_p
        _LIB.ref_project.restype = ctypes.c_int
        _LIB.ref_probe_texture.restype = ctypes.c_int
        _LIB.ref_probe_texture.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return _LIB


def available(n_volumes: int, n_materials: int, attenuate: bool = False) -> bool:
    return build_ref.cubin_path(n_volumes, n_materials, attenuate).exists()


def project(scene: Scene, *, solid_angle: bool = False, repeats: int = 0) -> dict:
    """Run the reference kernel on ``scene`` (its float32 geometry, tables and volumes)."""
    sc = scene.sc
    nv, M = sc.n_volumes, sc.n_materials
    path = build_ref.cubin_path(nv, M, bool(sc.attenuate_outside))
    if not path.exists():
        raise FileNotFoundError(f"reference cubin missing: {path}")
    if sc.attenuate_outside and sc.air_index != 0:
        raise ValueError("the reference cubins are built with AIR_INDEX=0")
    dens = (ctypes.c_void_p * nv)(*[sc.vol[i].density for i in range(nv)])
    labs = (ctypes.c_void_p * nv)(*[sc.vol[i].labels for i in range(nv)])
    dims = np.array([[sc.vol[i].ni, sc.vol[i].nj, sc.vol[i].nk] for i in range(nv)], dtype=np.int32)
    prio = np.array([sc.vol[i].priority for i in range(nv)], dtype=np.int32)
    en = np.array([sc.vol[i].enabled for i in range(nv)], dtype=np.int32)
    wfi = np.array(list(sc.world_from_index), dtype=np.float32)
    ijk = np.array([list(sc.vol[i].ijk_from_world) for i in range(nv)], dtype=np.float32)
    src = np.array([list(sc.vol[i].source_ijk) for i in range(nv)], dtype=np.float32)
    W, H = sc.width, sc.height
    inten = np.zeros((H, W), dtype=np.float32)
    prob = np.zeros((H, W), dtype=np.float32)
    sa = np.zeros((H, W), dtype=np.float32) if solid_angle else None
    ms = ctypes.c_float(0.0)
    L = lib()
    rc = L.ref_project(
        str(path).encode(), ctypes.c_int(nv), ctypes.c_int(M), dens, labs, dims.ctypes.data_as(ctypes.c_void_p),
        prio.ctypes.data_as(ctypes.c_void_p), en.ctypes.data_as(ctypes.c_void_p),
        wfi.ctypes.data_as(ctypes.c_void_p), ijk.ctypes.data_as(ctypes.c_void_p),
        src.ctypes.data_as(ctypes.c_void_p), ctypes.c_float(sc.max_ray_length), ctypes.c_float(sc.step),
        ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(sc.n_bins), ctypes.c_void_p(sc.energies),
        ctypes.c_void_p(sc.pdf), ctypes.c_void_p(sc.mu), ctypes.c_int(1 if solid_angle else 0),
        inten.ctypes.data_as(ctypes.c_void_p), prob.ctypes.data_as(ctypes.c_void_p),
        sa.ctypes.data_as(ctypes.c_void_p) if sa is not None else ctypes.c_void_p(0),
        ctypes.c_int(repeats), ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError("reference kernel harness: " + L.ref_last_error().decode())
    out = dict(intensity=inten, photon_prob=prob, ms=ms.value)
    if sa is not None:
        out["solid_angle"] = sa
    return out


def probe_texture(kind: int, volume_kji: np.ndarray, xyz: np.ndarray) -> np.ndarray:
    """Fetch the texture built from ``volume_kji`` ([nk][nj][ni]) at unnormalised coordinates
    ``xyz`` [n, 3]. kind 0: float32 linear; 1: uint8 point; 2: float16 linear."""
    dt = {0: np.float32, 1: np.uint8, 2: np.float16}[kind]
    vol = np.ascontiguousarray(volume_kji, dtype=dt)
    nk, nj, ni = vol.shape
    pts = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(pts.shape[0], dtype=np.float32)
    rc = lib().ref_probe_texture(kind, vol.ctypes.data, ni, nj, nk, pts.ctypes.data, pts.shape[0], out.ctypes.data)
    if rc != 0:
        raise RuntimeError("texture probe: " + lib().ref_last_error().decode())
    return out
