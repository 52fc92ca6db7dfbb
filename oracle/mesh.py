"""CPU restatement of the additive mesh pass: what the reference's OpenGL density pass
(deepdrr/pyrenderdrr/shaders/density.frag:9-13 with additive blending) and project_kernel.cu:569-579
contribute per pixel, under the rasterisation rules drr_mesh_area_density states. Test
infrastructure only.

Per triangle: vertices projected to index space (x - source through the inverse ray matrix,
perspective divide), snapped to 1/256 pixel; a pixel (u, v) is covered when its centre
(u + 0.5, v + 0.5) is inside by exact integer edge functions, ties going to top-left edges (an edge
P0 -> P1 of the positively oriented triangle owns its points when dy > 0, or dy == 0 and dx < 0).
A covered pixel adds sign * distance * density and sign, with distance the float64 intersection of
the pixel's unit ray with the triangle's plane and sign = +1 where the ray leaves along the
right-handed normal, -1 where it enters. The result per slot is max(R, 0) where |G| < 1e-5, else 0.
"""
from __future__ import annotations

import numpy as np


def _crossings(tri, W, Winv, s, width, height):
    """(triangle, u, v, distance, sign) arrays for each triangle that covers some pixel centre."""
    out = []
    for f in range(tri.shape[0]):
        P = tri[f]
        q = (P - s) @ Winv.T
        if not np.all(q[:, 2] > 1e-9):
            continue
        S = q[:, :2] / q[:, 2:3]
        if not np.all(np.abs(S) < 1.0e6):
            continue
        X = np.rint(S[:, 0] * 256.0).astype(np.int64)
        Y = np.rint(S[:, 1] * 256.0).astype(np.int64)
        area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0])
        if area == 0:
            continue
        o = [0, 1, 2] if area > 0 else [0, 2, 1]
        ax, ay, bx, by, cx, cy = X[o[0]], Y[o[0]], X[o[1]], Y[o[1]], X[o[2]], Y[o[2]]
        u0 = max((min(ax, bx, cx) - 128 + 255) >> 8, 0)
        u1 = min((max(ax, bx, cx) - 128) >> 8, width - 1)
        v0 = max((min(ay, by, cy) - 128 + 255) >> 8, 0)
        v1 = min((max(ay, by, cy) - 128) >> 8, height - 1)
        if u0 > u1 or v0 > v1:
            continue
        vv, uu = np.meshgrid(np.arange(v0, v1 + 1, dtype=np.int64), np.arange(u0, u1 + 1, dtype=np.int64),
                             indexing="ij")
        px, py = 256 * uu + 128, 256 * vv + 128

        def inside(x0, y0, x1, y1):
            e = (x1 - x0) * (py - y0) - (y1 - y0) * (px - x0)
            tl = (y1 - y0 > 0) or (y1 - y0 == 0 and x1 - x0 < 0)
            return (e > 0) | ((e == 0) & tl)

        cov = inside(ax, ay, bx, by) & inside(bx, by, cx, cy) & inside(cx, cy, ax, ay)
        if not cov.any():
            continue
        n = np.cross(P[1] - P[0], P[2] - P[0])
        npd = float(n @ (P[0] - s))
        fu, fv = uu[cov] + 0.5, vv[cov] + 0.5
        r = np.stack([fu, fv, np.ones_like(fu)], 1) @ W.T
        nr = (r @ n) / np.linalg.norm(r, axis=1)
        ok = nr != 0
        out.append((f, uu[cov][ok], vv[cov][ok], npd / nr[ok], np.where(nr[ok] > 0, 1.0, -1.0)))
    return out


def _view(world_from_index, source, triangles):
    W = np.asarray(world_from_index, dtype=np.float64).reshape(3, 3)
    return (W, np.linalg.inv(W), np.asarray(source, dtype=np.float64).reshape(3),
            np.asarray(triangles, dtype=np.float32).astype(np.float64).reshape(-1, 3, 3))


def hit_lists(triangles, layer, mode, n_layers: int, max_hits: int, world_from_index, source, width: int,
              height: int):
    """Subtractive crossings of one view: (alpha [L, H, W, K] float32, facing int8), sorted by
    distance, facing +1 entering and -1 leaving, 0 after the last (at most max_hits kept)."""
    W, Winv, s, tri = _view(world_from_index, source, triangles)
    lists = [[[[] for _ in range(width)] for _ in range(height)] for _ in range(n_layers)]
    for f, uu, vv, dist, sign in _crossings(tri, W, Winv, s, width, height):
        if not (int(mode[f]) & 2) or not (0 <= int(layer[f]) < n_layers):
            continue
        for u, v, d, g in zip(uu, vv, dist, sign):
            lists[int(layer[f])][v][u].append((np.float32(d), -1 if g > 0 else 1))
    A = np.zeros((n_layers, height, width, max_hits), np.float32)
    F = np.zeros((n_layers, height, width, max_hits), np.int8)
    for L in range(n_layers):
        for v in range(height):
            for u in range(width):
                h = sorted(lists[L][v][u], key=lambda x: x[0])[:max_hits]
                for k, (d, g) in enumerate(h):
                    A[L, v, u, k], F[L, v, u, k] = d, g
    return A, F


def mesh_area_density(triangles: np.ndarray, slot: np.ndarray, density: np.ndarray, n_slots: int,
                      world_from_index: np.ndarray, source: np.ndarray, width: int, height: int,
                      layer=None, mode=None, hits=None) -> np.ndarray:
    """[n_slots, H, W] float32 additive path integrals (mm g/cm^3) of one view. With `hits` (from
    hit_lists) the parts of a layer-l additive mesh inside the consecutive hit pairs of every layer
    above l are removed (density_between.frag)."""
    W, Winv, s, tri = _view(world_from_index, source, triangles)
    R = np.zeros((n_slots, height, width))
    G = np.zeros((n_slots, height, width))
    nF = tri.shape[0]
    layer = np.zeros(nF, np.int64) if layer is None else np.asarray(layer)
    mode = np.ones(nF, np.int64) if mode is None else np.asarray(mode)
    for f, uu, vv, dist, sign in _crossings(tri, W, Winv, s, width, height):
        if not (int(mode[f]) & 1):
            continue
        rho = float(density[f])
        add = sign * dist * rho
        if hits is not None:
            A, F = hits
            for L in range(int(layer[f]) + 1, A.shape[0]):
                for i in range(0, A.shape[3] - 1, 2):
                    pair_ok = (F[L, vv, uu, i] != 0) & (F[L, vv, uu, i + 1] != 0)
                    near = A[L, vv, uu, i].astype(np.float64)
                    far = A[L, vv, uu, i + 1].astype(np.float64)
                    g = np.where(dist < near, far - near, np.where(dist < far, far - dist, 0.0))
                    add = add + np.where(pair_ok, sign * rho * g, 0.0)
        np.add.at(R[int(slot[f])], (vv, uu), add)
        np.add.at(G[int(slot[f])], (vv, uu), sign)
    Rf, Gf = R.astype(np.float32), G.astype(np.float32)
    return np.where(np.abs(Gf) < 0.00001, np.maximum(Rf, 0.0), 0.0).astype(np.float32)
