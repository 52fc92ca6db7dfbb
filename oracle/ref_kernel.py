"""Python front end of ``ref_harness.cu``: runs the reference's own projectKernel on the GPU.

TEST AND BASELINE INFRASTRUCTURE ONLY (see ref_harness.cu): the GPU tests use it as the parity pin
and bench.py times it as the reference-kernel baseline. The cubins come from
``build_ref.build_cubins``; when they are absent (no reference sources where the tree was built)
``available`` is False and the tests that need them skip.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import build_ref
from .oracle import Scene, source_in_ijk

_LIB = None
MESH_LAYERS = 2      # the cubins' MESH_LAYERS (build_ref.py)
MAX_MESH_HITS = 32   # and MAX_MESH_HITS

_P = ctypes.c_void_p


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(str(build_ref.build_harness()))
        _LIB.ref_last_error.restype = ctypes.c_char_p
        _LIB.ref_project.restype = ctypes.c_int
        _LIB.ref_scene_create.restype = ctypes.c_int
        _LIB.ref_scene_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P,
                                          ctypes.c_int, _P, _P, _P, ctypes.POINTER(_P)]
        _LIB.ref_scene_destroy.restype = None
        _LIB.ref_scene_destroy.argtypes = [_P]
        _LIB.ref_scene_project.restype = ctypes.c_int
        _LIB.ref_scene_project.argtypes = [_P, _P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_int, _P, _P,
                                           _P, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                           ctypes.POINTER(ctypes.c_float)]
        _LIB.ref_probe_texture.restype = ctypes.c_int
        _LIB.ref_probe_texture.argtypes = [ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P,
                                           ctypes.c_int, _P]
    return _LIB


def available(n_volumes: int, n_materials: int, attenuate: bool = False, mesh_additive: bool = False) -> bool:
    return build_ref.cubin_path(n_volumes, n_materials, attenuate, mesh_additive).exists()


def _ptr(a: Optional[np.ndarray]):
    return _P(0) if a is None else _P(a.ctypes.data)


class RefScene:
    """The reference kernel with its textures and tables resident, like an initialised Projector.

    ``volumes``: dicts with ``density`` float32 [ni, nj, nk], ``labels`` uint8 (index into the
    sorted material list) and ``ijk_from_world`` (3x4 or 4x4 float64); ``energies`` / ``pdf`` /
    ``mu`` [n_bins][M] float32 as the projector uploads them."""

    def __init__(self, volumes: Sequence[dict], *, energies, pdf, mu, priorities=None, enabled=None,
                 attenuate: bool = False, mesh_additive: bool = False):
        nv = len(volumes)
        mu = np.ascontiguousarray(mu, dtype=np.float32)
        n_bins, M = mu.shape
        path = build_ref.cubin_path(nv, M, attenuate, mesh_additive)
        if not path.exists():
            raise FileNotFoundError(f"reference cubin missing: {path}")
        self.n_volumes, self.n_materials = nv, M
        dens = [np.ascontiguousarray(np.asarray(v["density"], np.float32).transpose(2, 1, 0)) for v in volumes]
        labs = [np.ascontiguousarray(np.asarray(v["labels"], np.uint8).transpose(2, 1, 0)) for v in volumes]
        self.ijk_from_world = []
        for v in volumes:
            A = np.asarray(v["ijk_from_world"], dtype=np.float64)
            self.ijk_from_world.append(A if A.shape == (4, 4) else np.vstack([A[:3, :4], [0, 0, 0, 1]]))
        dims = np.array([list(np.asarray(v["density"]).shape) for v in volumes], dtype=np.int32)
        prio = np.array(priorities if priorities is not None else [nv - 1 - i for i in range(nv)], dtype=np.int32)
        en = np.array(enabled if enabled is not None else [1] * nv, dtype=np.int32)
        e = np.ascontiguousarray(energies, dtype=np.float32)
        p = np.ascontiguousarray(pdf, dtype=np.float32)
        dp = (_P * nv)(*[d.ctypes.data for d in dens])
        lp = (_P * nv)(*[l.ctypes.data for l in labs])
        h = _P(0)
        L = lib()
        rc = L.ref_scene_create(str(path).encode(), nv, M, ctypes.cast(dp, _P), ctypes.cast(lp, _P), _ptr(dims),
                                _ptr(prio), _ptr(en), n_bins, _ptr(e), _ptr(p), _ptr(mu), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("reference kernel harness: " + L.ref_last_error().decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().ref_scene_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def view_arrays(self, world_from_index, source_world):
        """The float32 geometry _update_object_locations uploads (projector.py:802-831)."""
        w = np.asarray(world_from_index, dtype=np.float64)[:3, :3].astype(np.float32).ravel()
        ijk = np.stack([A[:3, :4].astype(np.float32).ravel() for A in self.ijk_from_world])
        src = np.stack([source_in_ijk(A, source_world).astype(np.float32) for A in self.ijk_from_world])
        return np.ascontiguousarray(w), np.ascontiguousarray(ijk), np.ascontiguousarray(src)

    def project(self, world_from_index, source_world, width: int, height: int, *, step: float,
                max_ray_length: float = -4.0, solid_angle: bool = False, outputs: bool = True, repeats: int = 0,
                wall: bool = False, hit_alpha=None, hit_facing=None, layer_valid=None, additive=None,
                unique_materials=None) -> dict:
        """One view. Mesh inputs in the reference's layouts: hit lists [2][H][W][32] (float32 /
        int8) with ``layer_valid`` [2]; additive densities [2][n_umat][H][W][2] with
        ``unique_materials`` [n_umat] (needs a scene built with ``mesh_additive``)."""
        w, ijk, src = self.view_arrays(world_from_index, source_world)
        H, W = int(height), int(width)
        inten = np.zeros((H, W), np.float32) if outputs else None
        prob = np.zeros((H, W), np.float32) if outputs else None
        sa = np.zeros((H, W), np.float32) if (outputs and solid_angle) else None
        ha = hf = lv = ad = um = None
        if hit_alpha is not None:
            shape = (MESH_LAYERS, H, W, MAX_MESH_HITS)
            ha = np.ascontiguousarray(hit_alpha, np.float32)
            hf = np.ascontiguousarray(hit_facing, np.int8)
            lv = np.ascontiguousarray(layer_valid, np.int8)
            if ha.shape != shape or hf.shape != shape or lv.shape != (MESH_LAYERS,):
                raise ValueError(f"hit lists must be {shape} with layer_valid [{MESH_LAYERS}]")
        n_umat = 0
        if additive is not None:
            ad = np.ascontiguousarray(additive, np.float32)
            um = np.ascontiguousarray(unique_materials, np.int32)
            n_umat = int(um.shape[0])
            if ad.shape != (MESH_LAYERS, n_umat, H, W, 2):
                raise ValueError("additive densities must be [2][n_umat][H][W][2]")
        ms, wall_ms = ctypes.c_float(0.0), ctypes.c_float(0.0)
        L = lib()
        rc = L.ref_scene_project(self._h, _ptr(w), _ptr(ijk), _ptr(src), float(max_ray_length), float(step), W, H,
                                 1 if solid_angle else 0, _ptr(ha), _ptr(hf), _ptr(lv), _ptr(ad), _ptr(um), n_umat,
                                 _ptr(inten), _ptr(prob), _ptr(sa), int(repeats), ctypes.byref(ms),
                                 ctypes.byref(wall_ms) if wall else None)
        if rc != 0:
            raise RuntimeError("reference kernel harness: " + L.ref_last_error().decode())
        out = dict(ms=ms.value)
        if wall:
            out["wall_ms"] = wall_ms.value
        if outputs:
            out.update(intensity=inten, photon_prob=prob)
            if sa is not None:
                out["solid_angle"] = sa
        return out


def project(scene: Scene, *, solid_angle: bool = False, repeats: int = 0) -> dict:
    """Run the reference kernel on ``scene`` (its float32 geometry, tables and volumes)."""
    sc = scene.sc
    nv, M = sc.n_volumes, sc.n_materials
    path = build_ref.cubin_path(nv, M, bool(sc.attenuate_outside))
    if not path.exists():
        raise FileNotFoundError(f"reference cubin missing: {path}")
    if sc.attenuate_outside and sc.air_index != 0:
        raise ValueError("the reference cubins are built with AIR_INDEX=0")
    dens = (_P * nv)(*[sc.vol[i].density for i in range(nv)])
    labs = (_P * nv)(*[sc.vol[i].labels for i in range(nv)])
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
        str(path).encode(), ctypes.c_int(nv), ctypes.c_int(M), dens, labs, dims.ctypes.data_as(_P),
        prio.ctypes.data_as(_P), en.ctypes.data_as(_P), wfi.ctypes.data_as(_P), ijk.ctypes.data_as(_P),
        src.ctypes.data_as(_P), ctypes.c_float(sc.max_ray_length), ctypes.c_float(sc.step),
        ctypes.c_int(W), ctypes.c_int(H), ctypes.c_int(sc.n_bins), _P(sc.energies), _P(sc.pdf), _P(sc.mu),
        ctypes.c_int(1 if solid_angle else 0), inten.ctypes.data_as(_P), prob.ctypes.data_as(_P),
        sa.ctypes.data_as(_P) if sa is not None else _P(0), ctypes.c_int(repeats), ctypes.byref(ms))
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
