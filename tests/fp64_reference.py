"""Float64 torch restatement of the single-volume forward projection, differentiable by autograd:
the reference for the adjoint's density and pose gradients.

It follows the reference kernel's algorithm for one volume without air attenuation
(deepdrr/projector/project_kernel.cu:218-646): unit ray per pixel, slab test in IJK, steps
alpha_t = minAlpha + t * step from minAlpha = min(|r|, entry) with the -1 voxel offset, trapezoid
half weights at t = 0 and t = num_steps - 1, samples only inside the volume's interval, trilinear
label fractions, density from the texture filter, path lengths x step / 10, and the polychromatic
Beer-Lambert sum. Arithmetic is float64 (no float32 alpha drift). The step grid (which steps are
sampled, and their weights) is taken from the unmoved pose and held fixed, as the adjoint does.

filter="hw": the texture unit's 8-bit corner weights (piecewise constant in position: gradients
flow to the densities only); filter="exact": exact trilinear weights (gradients to densities and
positions).
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _rotation(w):
    th = torch.sqrt((w * w).sum() + 1e-300)
    z = torch.zeros((), dtype=w.dtype)
    K = torch.stack([torch.stack([z, -w[2], w[1]]), torch.stack([w[2], z, -w[0]]), torch.stack([-w[1], w[0], z])])
    eye = torch.eye(3, dtype=w.dtype)
    if float(th.detach()) < 1e-8:
        return eye + K + 0.5 * K @ K
    return eye + torch.sin(th) / th * K + (1.0 - torch.cos(th)) / (th * th) * K @ K


def rigid_motion_t(pose, center):
    """4x4 Translate(center + t) R(w) Translate(-center) as a differentiable torch float64 matrix."""
    c = torch.as_tensor(np.asarray(center, dtype=np.float64))
    R = _rotation(pose[3:])
    top = torch.cat([R, (c + pose[:3] - R @ c)[:, None]], 1)
    return torch.cat([top, torch.tensor([[0.0, 0.0, 0.0, 1.0]], dtype=torch.float64)], 0)


def _hw_axis(x, n):
    xb = torch.clamp(x - 0.5, 0.0, n - 1.0)
    fix = torch.floor(xb * 256.0 + 0.5).long()
    i0 = fix >> 8
    return i0, torch.clamp(i0 + 1, max=n - 1), fix & 255


def _hw_weights(Ax, Ay, Az):
    """The texture unit's corner weights (units of 1/256), corner c = dx | dy << 1 | dz << 2."""
    W = [None] * 8
    for dz in (0, 1):
        vz = Az if dz else 256 - Az
        hx = (vz * Ax + 128) >> 8
        for dx in (0, 1):
            vx = hx if dx else vz - hx
            hy = (vx * Ay + 128) >> 8 if dx else vx - ((vx * (256 - Ay) + 128) >> 8)
            W[dx | 2 | (dz << 2)] = hy
            W[dx | (dz << 2)] = vx - hy
    return W


def project_fp64(density, labels, ijk0, world_from_index, source_world, width, height, step, energies, pdf, mu,
                 pose=None, center=None, filter="exact"):
    """intensity, photon_prob [H, W] and area densities [M, H, W] (float64 torch) of one view.

    density: torch float64 [ni, nj, nk] (may require grad); labels: numpy uint8 [ni, nj, nk];
    ijk0: 4x4 IJK_from_world of the unmoved volume; pose: optional torch (6,) float64."""
    ni, nj, nk = labels.shape
    M = mu.shape[1]
    W = np.asarray(world_from_index, dtype=np.float64)[:3, :3]
    src = np.asarray(source_world, dtype=np.float64)
    A0 = np.asarray(ijk0, dtype=np.float64)
    # step grid from the unmoved pose
    vv, uu = np.meshgrid(np.arange(height) + 0.5, np.arange(width) + 0.5, indexing="ij")
    pix = np.stack([uu.ravel(), vv.ravel(), np.ones(uu.size)], 1)
    r = pix @ W.T
    ray_length = np.linalg.norm(r, axis=1)
    r = r / ray_length[:, None]
    s0 = A0[:3, :3] @ src + A0[:3, 3]
    rd0 = r @ A0[:3, :3].T
    hi = np.array([ni - 0.5, nj - 0.5, nk - 0.5])
    with np.errstate(divide="ignore", invalid="ignore"):
        a0 = (-0.5 - s0[None, :]) / rd0
        a1 = (hi[None, :] - s0[None, :]) / rd0
    inside = (s0[None, :] >= -0.5) & (s0[None, :] <= hi[None, :])
    lo_a = np.where(rd0 != 0, np.minimum(a0, a1), np.where(inside, -np.inf, np.inf))
    hi_a = np.where(rd0 != 0, np.maximum(a0, a1), np.where(inside, np.inf, -np.inf))
    mn = np.maximum(0.0, lo_a.max(1))
    mx = hi_a.min(1)
    minA = np.minimum(ray_length, mn)
    maxA = np.maximum(0.0, mx)
    num_steps = np.ceil((maxA - minA) / step).astype(np.int64)
    T = int(max(num_steps.max(), 1))
    t = np.arange(T)[None, :]
    alpha = minA[:, None] + t * step
    live = (t < num_steps[:, None]) & (alpha >= mn[:, None]) & (alpha <= mx[:, None]) & (mn <= mx)[:, None]
    wt = np.where((t == 0) | (t == num_steps[:, None] - 1), 0.5, 1.0) * live
    ray_i, step_i = np.nonzero(live)
    # positions, differentiable in the pose
    A = torch.as_tensor(A0)
    if pose is not None:
        A = A @ torch.linalg.inv(rigid_motion_t(pose, center))
    x = torch.as_tensor(src)[None, :] + torch.as_tensor(alpha[ray_i, step_i])[:, None] * torch.as_tensor(r[ray_i])
    p = x @ A[:3, :3].T + A[:3, 3][None, :] - 1.0
    w_t = torch.as_tensor(wt[ray_i, step_i])
    base = torch.floor(p.detach())
    f = p - base
    b = base.long()
    n = torch.tensor([ni, nj, nk])
    dens = density
    lab = torch.as_tensor(labels.astype(np.int64))
    seg = torch.zeros((p.shape[0], M), dtype=torch.float64)
    rho = torch.zeros(p.shape[0], dtype=torch.float64)
    if filter == "hw":
        xs = p.detach() + 0.5
        i0, i1, Ax = _hw_axis(xs[:, 0], ni)
        j0, j1, Ay = _hw_axis(xs[:, 1], nj)
        k0, k1, Az = _hw_axis(xs[:, 2], nk)
        Wc = _hw_weights(Ax, Ay, Az)
        ii, jj, kk = (i0, i1), (j0, j1), (k0, k1)
    for c in range(8):
        d = torch.tensor([c & 1, (c >> 1) & 1, c >> 2])
        idx = torch.minimum(torch.clamp(b + d[None, :], min=0), n[None, :] - 1)
        wx = f[:, 0] if c & 1 else 1.0 - f[:, 0]
        wy = f[:, 1] if (c >> 1) & 1 else 1.0 - f[:, 1]
        wz = f[:, 2] if c >> 2 else 1.0 - f[:, 2]
        w = wx * wy * wz
        L = lab[idx[:, 0], idx[:, 1], idx[:, 2]]
        seg = seg + torch.nn.functional.one_hot(L, M).double() * w[:, None]
        if filter == "hw":
            rho = rho + Wc[c].double() / 256.0 * dens[ii[c & 1], jj[(c >> 1) & 1], kk[c >> 2]]
        else:
            rho = rho + w * dens[idx[:, 0], idx[:, 1], idx[:, 2]]
    contrib = (w_t * rho)[:, None] * seg
    raw = torch.zeros((height * width, M), dtype=torch.float64).index_add(0, torch.as_tensor(ray_i), contrib)
    ad = raw * step / 10.0
    mu_t = torch.as_tensor(np.asarray(mu, dtype=np.float64))
    e = torch.exp(-(ad @ mu_t.T)) * torch.as_tensor(np.asarray(pdf, dtype=np.float64))[None, :]
    inten = e @ torch.as_tensor(np.asarray(energies, dtype=np.float64))
    prob = e.sum(1)
    return inten.reshape(height, width), prob.reshape(height, width), ad.T.reshape(M, height, width)


def project_fp64_at_samples(density, labels, ijk_at, samples, width, height, step, energies, pdf, mu,
                            pose=None, ijk0=None, center=None, filter="exact"):
    """The same projection evaluated at given sample positions: the float32 positions the product
    (and the float32 oracle, which reproduces them bit for bit) takes along each ray.

    ijk_at: 4x4 IJK_from_world the samples were taken with; samples: per ray (row-major) a tuple
    (alpha [n], p [n, 3], weight [n]) from oracle.Scene.ray_samples. With `pose` (torch (6,)
    float64) the volume is IJK_from_world(pose) = ijk0 . inv(rigid_motion(pose, center)) and a
    sample at world point x sits at p + (IJK_from_world(pose) - ijk_at) x: equal to p where pose
    gives ijk_at, with the exact derivative there. Returns intensity, photon_prob [H, W] and area
    densities [M, H, W] (float64 torch)."""
    ni, nj, nk = labels.shape
    M = mu.shape[1]
    At = np.asarray(ijk_at, dtype=np.float64)
    counts = [len(s[0]) for s in samples]
    ray_i = np.repeat(np.arange(len(samples)), counts)
    P32 = np.concatenate([s[1] for s in samples]).astype(np.float64) if ray_i.size else np.zeros((0, 3))
    W32 = np.concatenate([s[2] for s in samples]).astype(np.float64) if ray_i.size else np.zeros(0)
    # world points of the samples
    x = (P32 + 1.0 - At[:3, 3][None, :]) @ np.linalg.inv(At[:3, :3]).T
    p = torch.as_tensor(P32)
    if pose is not None:
        A = torch.as_tensor(np.asarray(ijk0, dtype=np.float64)) @ torch.linalg.inv(rigid_motion_t(pose, center))
        dA = A - torch.as_tensor(At)
        p = p + torch.as_tensor(x) @ dA[:3, :3].T + dA[:3, 3][None, :]
    base = torch.as_tensor(np.floor(P32))
    f = p - base
    b = base.long()
    n = torch.tensor([ni, nj, nk])
    lab = torch.as_tensor(labels.astype(np.int64))
    seg = torch.zeros((p.shape[0], M), dtype=torch.float64)
    rho = torch.zeros(p.shape[0], dtype=torch.float64)
    if filter == "hw":
        tx = torch.as_tensor((np.concatenate([s[1] for s in samples]) + np.float32(0.5)).astype(np.float64))
        i0, i1, Ax = _hw_axis(tx[:, 0], ni)
        j0, j1, Ay = _hw_axis(tx[:, 1], nj)
        k0, k1, Az = _hw_axis(tx[:, 2], nk)
        Wc = _hw_weights(Ax, Ay, Az)
        ii, jj, kk = (i0, i1), (j0, j1), (k0, k1)
    for c in range(8):
        d = torch.tensor([c & 1, (c >> 1) & 1, c >> 2])
        idx = torch.minimum(torch.clamp(b + d[None, :], min=0), n[None, :] - 1)
        wx = f[:, 0] if c & 1 else 1.0 - f[:, 0]
        wy = f[:, 1] if (c >> 1) & 1 else 1.0 - f[:, 1]
        wz = f[:, 2] if c >> 2 else 1.0 - f[:, 2]
        w = wx * wy * wz
        L = lab[idx[:, 0], idx[:, 1], idx[:, 2]]
        seg = seg + torch.nn.functional.one_hot(L, M).double() * w[:, None]
        if filter == "hw":
            rho = rho + Wc[c].double() / 256.0 * density[ii[c & 1], jj[(c >> 1) & 1], kk[c >> 2]]
        else:
            rho = rho + w * density[idx[:, 0], idx[:, 1], idx[:, 2]]
    contrib = (torch.as_tensor(W32) * rho)[:, None] * seg
    raw = torch.zeros((height * width, M), dtype=torch.float64).index_add(0, torch.as_tensor(ray_i), contrib)
    ad = raw * float(np.float32(step)) / 10.0
    mu_t = torch.as_tensor(np.asarray(mu, dtype=np.float64))
    e = torch.exp(-(ad @ mu_t.T)) * torch.as_tensor(np.asarray(pdf, dtype=np.float64))[None, :]
    inten = e @ torch.as_tensor(np.asarray(energies, dtype=np.float64))
    prob = e.sum(1)
    return inten.reshape(height, width), prob.reshape(height, width), ad.T.reshape(M, height, width)
