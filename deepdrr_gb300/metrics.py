"""Work accounting for the benchmark: samples and algorithmic bytes.

A *sample* is one (ray, step t, volume i) with volume i live at that step: traced, enabled, and
alpha_t = minAlpha + t * step inside [minAlpha_i, maxAlpha_i] (the range test of
deepdrr/projector/project_kernel.cu:472). Samples are counted in float64 in closed form per ray
and volume from the same slab test as the kernel (project_kernel.cu:265-334).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

from . import geo

# Bytes the march reads per sample: 8 density texels and 8 label texels (one trilinear neighbourhood).
BYTES_PER_SAMPLE = {"float32": 8 * 4 + 8 * 1, "float16": 8 * 2 + 8 * 1, "bfloat16": 8 * 2 + 8 * 1}


def count_samples(volumes, projs, step: float, max_ray_length: float = -1.0, device: str = "cpu") -> np.ndarray:
    """Number of live samples per view (float64 closed form)."""
    import torch

    out = []
    for proj in projs:
        W, src, w, h = geo.view_arrays(proj)
        Wt = torch.tensor(W, dtype=torch.float64, device=device)
        u = torch.arange(w, dtype=torch.float64, device=device) + 0.5
        v = torch.arange(h, dtype=torch.float64, device=device) + 0.5
        vv, uu = torch.meshgrid(v, u, indexing="ij")
        r = torch.stack([uu, vv, torch.ones_like(uu)], -1) @ Wt.T  # [h, w, 3]
        rl = torch.linalg.norm(r, dim=-1)
        rd = r / rl[..., None]
        minA = rl.clone()
        maxA = torch.zeros_like(rl)
        per_vol = []
        for vol in volumes:
            if not vol.enabled:
                continue
            A = torch.tensor(np.asarray(vol.ijk_from_world.data)[:3, :4], dtype=torch.float64, device=device)
            s = A[:, :3] @ torch.tensor(src, dtype=torch.float64, device=device) + A[:, 3]
            ri = rd @ A[:, :3].T
            mn = torch.zeros_like(rl)
            mx = torch.full_like(rl, max_ray_length if max_ray_length > 0 else float("inf"))
            ok = torch.ones_like(rl, dtype=torch.bool)
            for ax, n in enumerate(vol.shape):
                ra = ri[..., ax]
                nz = ra != 0
                a0 = (-0.5 - s[ax]) / torch.where(nz, ra, torch.ones_like(ra))
                a1 = (n - 0.5 - s[ax]) / torch.where(nz, ra, torch.ones_like(ra))
                mn = torch.where(nz, torch.maximum(mn, torch.minimum(a0, a1)), mn)
                mx = torch.where(nz, torch.minimum(mx, torch.maximum(a0, a1)), mx)
                inside = (-0.5 <= s[ax]) & (s[ax] <= n - 0.5)
                ok = ok & (nz | inside)
            minA = torch.where(ok, torch.minimum(minA, mn), minA)
            maxA = torch.where(ok, torch.maximum(maxA, mx), maxA)
            per_vol.append((ok, mn, mx))
        ns = torch.clamp(torch.ceil((maxA - minA) / step), min=0)
        total = torch.zeros((), dtype=torch.float64, device=device)
        for ok, mn, mx in per_vol:
            t0 = torch.clamp(torch.ceil((mn - minA) / step), min=0)
            t1 = torch.minimum(torch.floor((mx - minA) / step), ns - 1)
            cnt = torch.clamp(t1 - t0 + 1, min=0)
            total = total + torch.where(ok & (mn <= mx), cnt, torch.zeros_like(cnt)).sum()
        out.append(float(total))
    return np.asarray(out)


def compulsory_bytes(volumes, width: int, height: int, density_dtype: str = "float32", outputs: int = 2) -> int:
    """Bytes one view must move at least once through HBM: every voxel's density and label, plus
    the float32 output images."""
    db = {"float32": 4, "float16": 2, "bfloat16": 2}[density_dtype]
    vox = sum(int(np.prod(v.shape)) for v in volumes)
    return vox * (db + 1) + width * height * 4 * outputs
