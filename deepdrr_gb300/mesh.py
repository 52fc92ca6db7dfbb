"""Triangle meshes that add their material's path length to the projection.

Restates what the projector reads from the reference's mesh renderables (deepdrr/vol/mesh.py:40-186
with deepdrr/pyrenderdrr/material.py): triangles with a pose, a material name and a density
(g/cm^3; defaults from the reference's DRRMaterial table), and whether the mesh is additive. The
reference renders meshes with OpenGL; this package rasterises them in CUDA (drr_mesh_area_density).

A subtractive mesh (``subtractive=True``) removes, along each ray, the volumes' samples inside it
and the parts of additive meshes of lower layers inside it (the reference's MESH_SUB pass); an
additive one adds its material's path length. A mesh can be both, as a reference material can.
"""
from __future__ import annotations

import struct
from pathlib import Path
from typing import Optional, Tuple, Union

import numpy as np

from .geo import FrameTransform

__all__ = ["Mesh", "DEFAULT_DENSITIES", "read_stl"]

# g/cm^3, the reference's DRRMaterial._default_densities (pyrenderdrr/material.py)
DEFAULT_DENSITIES = {
    "bone": 1.92, "soft tissue": 1.0, "tissue_soft": 1.0, "blood": 1.06, "muscle": 1.06, "air": 0.0012,
    "iron": 7.87, "lead": 11.34, "copper": 8.96, "lung": 0.26, "titanium": 4.51, "teflon": 2.2,
    "polyethylene": 0.94, "concrete": 2.3,
}


def read_stl(path: Union[str, Path]) -> Tuple[np.ndarray, np.ndarray]:
    """(vertices [V, 3] float64, faces [F, 3] int64) of a binary or ASCII STL file (vertices are
    not merged: each facet has its own three)."""
    data = Path(path).read_bytes()
    if len(data) >= 84:
        n = struct.unpack_from("<I", data, 80)[0]
        if 84 + 50 * n == len(data):
            rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]),
                                count=n, offset=84)
            verts = rec["v"].reshape(-1, 3).astype(np.float64)
            return verts, np.arange(3 * n, dtype=np.int64).reshape(n, 3)
    verts = []
    for line in data.decode("ascii", "replace").splitlines():
        tok = line.split()
        if len(tok) == 4 and tok[0] == "vertex":
            verts.append([float(t) for t in tok[1:]])
    if not verts or len(verts) % 3:
        raise ValueError(f"{path}: not a binary or ASCII STL file")
    v = np.asarray(verts, dtype=np.float64)
    return v, np.arange(len(v), dtype=np.int64).reshape(-1, 3)


class Mesh:
    """A closed triangle surface of one material, wound so its right-handed normals point out."""

    def __init__(self, vertices: np.ndarray, faces: np.ndarray, material: str = "iron",
                 density: Optional[float] = None, additive: bool = True, subtractive: bool = False,
                 layer: int = 0, world_from_anatomical: Optional[FrameTransform] = None, enabled: bool = True):
        if not (additive or subtractive):
            raise ValueError("a mesh must be additive, subtractive or both")
        self.additive = bool(additive)
        self.subtractive = bool(subtractive)
        self.layer = int(layer)
        if self.layer < 0:
            raise ValueError("layer must be >= 0")
        self.vertices = np.asarray(vertices, dtype=np.float64).reshape(-1, 3)
        self.faces = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
        if self.faces.size and (self.faces.min() < 0 or self.faces.max() >= len(self.vertices)):
            raise ValueError("face index outside the vertex array")
        self.material = str(material)
        if density is None:
            if self.material not in DEFAULT_DENSITIES:
                raise ValueError(f"no default density for {material!r}; pass density=")
            density = DEFAULT_DENSITIES[self.material]
        if density < 0:
            raise ValueError("density must be >= 0")
        self.density = float(density)
        self.world_from_anatomical = FrameTransform(world_from_anatomical)
        self.enabled = bool(enabled)

    @classmethod
    def from_stl(cls, path: Union[str, Path], material: str = "iron", **kwargs) -> "Mesh":
        v, f = read_stl(path)
        return cls(v, f, material=material, **kwargs)

    @classmethod
    def box(cls, size=(10.0, 10.0, 10.0), center=(0.0, 0.0, 0.0), **kwargs) -> "Mesh":
        """An axis-aligned box (12 outward-wound triangles)."""
        h = np.asarray(size, dtype=np.float64) / 2
        c = np.asarray(center, dtype=np.float64)
        v = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], dtype=np.float64) * h + c
        # vertex index = 4 x + 2 y + z with x, y, z in {0, 1}
        f = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5],   # x = -, x = +
                      [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],   # y = -, y = +
                      [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]])  # z = -, z = +
        return cls(v, f, **kwargs)

    @classmethod
    def icosphere(cls, radius: float = 10.0, center=(0.0, 0.0, 0.0), subdivisions: int = 3, **kwargs) -> "Mesh":
        """A sphere from a subdivided icosahedron, outward-wound."""
        t = (1.0 + 5 ** 0.5) / 2
        v = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
             [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
        f = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
             [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11],
             [6, 2, 10], [8, 6, 7], [9, 8, 1]]
        verts = [np.asarray(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
        faces = f
        for _ in range(subdivisions):
            cache = {}

            def mid(a, b):
                key = (min(a, b), max(a, b))
                if key not in cache:
                    m = verts[a] + verts[b]
                    verts.append(m / np.linalg.norm(m))
                    cache[key] = len(verts) - 1
                return cache[key]

            nf = []
            for a, b, c in faces:
                ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
                nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
            faces = nf
        V = np.asarray(verts) * float(radius) + np.asarray(center, dtype=np.float64)
        return cls(V, np.asarray(faces, dtype=np.int64), **kwargs)

    def triangles_in_world(self) -> np.ndarray:
        """[F, 3, 3] float64 triangle vertices in world coordinates."""
        T = self.world_from_anatomical.data
        w = self.vertices @ T[:3, :3].T + T[:3, 3]
        return w[self.faces]

    def translate(self, t) -> "Mesh":
        self.world_from_anatomical = FrameTransform.from_rt(translation=np.asarray(t, dtype=np.float64)) \
            @ self.world_from_anatomical
        return self

    def __repr__(self) -> str:
        return f"Mesh({len(self.faces)} triangles, material={self.material!r}, density={self.density})"
