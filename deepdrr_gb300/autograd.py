"""Differentiable projection: ``torch.autograd.Function`` over ``drr_project`` / ``drr_project_adjoint``.

The reference projector is not differentiable (deepdrr README.md:47); this module adds gradients
of the projection of one volume with respect to its densities and to a rigid motion of the volume
(6-DoF: translation t and rotation vector w, the volume turned about ``center`` and then moved by
t, in world coordinates):

    world_from_ijk(theta) = Translate(center + t) . R(w) . Translate(-center) . world_from_ijk

The library returns the derivative with respect to a small extra motion applied on top of the
current one, about the moved centre; the chain rule to (t, w) is exact: dL/dt is that translation
derivative and dL/dw = J_l(w)^T times the rotation derivative, J_l the left Jacobian of SO(3).
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np

from .projector import Projector

__all__ = ["rotation", "left_jacobian", "rigid_motion", "project"]


def _skew(w) -> np.ndarray:
    x, y, z = (float(c) for c in w)
    return np.array([[0.0, -z, y], [z, 0.0, -x], [-y, x, 0.0]])


def rotation(w) -> np.ndarray:
    """Rodrigues' formula: the rotation matrix of rotation vector ``w`` (radians)."""
    w = np.asarray(w, dtype=np.float64)
    th = float(np.linalg.norm(w))
    K = _skew(w)
    if th < 1e-8:
        return np.eye(3) + K + 0.5 * K @ K
    return np.eye(3) + math.sin(th) / th * K + (1.0 - math.cos(th)) / th ** 2 * K @ K


def left_jacobian(w) -> np.ndarray:
    """J_l(w): exp((w + dw)^) = exp((J_l(w) dw)^) exp(w^) to first order."""
    w = np.asarray(w, dtype=np.float64)
    th = float(np.linalg.norm(w))
    K = _skew(w)
    if th < 1e-6:
        return np.eye(3) + 0.5 * K + K @ K / 6.0
    return np.eye(3) + (1.0 - math.cos(th)) / th ** 2 * K + (th - math.sin(th)) / th ** 3 * K @ K


def rigid_motion(pose, center) -> np.ndarray:
    """4x4 world transform Translate(center + t) R(w) Translate(-center) of pose (t, w)."""
    pose = np.asarray(pose, dtype=np.float64).reshape(6)
    c = np.asarray(center, dtype=np.float64).reshape(3)
    T = np.eye(4)
    R = rotation(pose[3:])
    T[:3, :3] = R
    T[:3, 3] = c + pose[:3] - R @ c
    return T


class _State:
    def __init__(self, projector: Projector, cams, center, recompute: bool, want_area_density: bool,
                 distributed: bool = False, group=None):
        self.distributed = distributed
        self.group = group
        self.projector = projector
        self.cams = cams
        self.center = np.asarray(center, dtype=np.float64)
        self.recompute = recompute
        self.want_area_density = want_area_density
        v = projector.volumes[0]
        self.ijk0 = np.asarray(v.ijk_from_world.data, dtype=np.float64)

    def ijk_from_world(self, pose_np) -> np.ndarray:
        if pose_np is None:
            return self.ijk0[None, :3, :4]
        return (self.ijk0 @ np.linalg.inv(rigid_motion(pose_np, self.center)))[None, :3, :4]


def _function():
    import torch

    class _Project(torch.autograd.Function):
        @staticmethod
        def forward(ctx, density, pose, state: _State):
            ctx.set_materialize_grads(False)
            proj = state.projector
            if density is not None:
                proj.set_density(density)
            pose_np = None if pose is None else pose.detach().cpu().double().numpy()
            ijk = state.ijk_from_world(pose_np)
            keep_ad = state.want_area_density or not state.recompute
            out = proj.project_tensors(*state.cams, area_density=keep_ad, ijk_from_world=ijk)
            ctx.state = state
            ctx.pose_np = pose_np
            ctx.ijk = ijk
            ctx.pose_meta = None if pose is None else (pose.device, pose.dtype)
            ctx.density_given = density is not None
            ctx.save_for_backward(density if density is not None else None)
            ctx.area_density = None if state.recompute else out["area_density"].detach()
            ad = out["area_density"] if state.want_area_density else out["intensity"].new_empty(0)
            return out["intensity"], out["photon_prob"], ad

        @staticmethod
        def backward(ctx, g_int, g_prob, g_ad):
            state = ctx.state
            proj = state.projector
            (density,) = ctx.saved_tensors
            if g_ad is not None and g_ad.numel() == 0:
                g_ad = None
            if ctx.density_given:
                proj.set_density(density)  # the texture may hold a later iterate
            want_d = ctx.needs_input_grad[0]
            want_p = ctx.needs_input_grad[1]
            if not (want_d or want_p) or (g_int is None and g_prob is None and g_ad is None):
                return None, None, None
            c = state.center if ctx.pose_np is None else state.center + ctx.pose_np[:3]
            r = proj.project_adjoint(
                *state.cams, area_density=ctx.area_density,
                grad_intensity=None if g_int is None else g_int.contiguous().float(),
                grad_photon_prob=None if g_prob is None else g_prob.contiguous().float(),
                grad_area_density=None if g_ad is None else g_ad.contiguous().float(),
                density=want_d, pose=want_p, center=c, ijk_from_world=ctx.ijk)
            gd = r["density"].contiguous() if want_d else None
            gp = None
            if state.distributed:
                # each rank back-projected its own views: the shared parameters' gradients are sums
                from .replicas import sum_gradient_

                if gd is not None:
                    sum_gradient_(gd, state.group)
                if want_p:
                    pose_sum = r["pose"].double().sum(0).cpu()
                    sum_gradient_(pose_sum, state.group)
                    r["pose"] = pose_sum[None]
            if want_p:
                g = r["pose"].double().sum(0).cpu().numpy()
                g[3:] = left_jacobian(ctx.pose_np[3:]).T @ g[3:]
                dev, dt = ctx.pose_meta
                gp = torch.from_numpy(g).to(device=dev, dtype=dt)
            return gd, gp, None

    return _Project


_PROJECT = None


def project(projector: Projector, *camera_projections, density=None, pose=None, center=None,
            recompute: bool = False, area_density: bool = False, distributed: bool = False, group=None) -> dict:
    """Differentiable projection of the projector's single volume.

    ``density``: optional CUDA float32 tensor [ni, nj, nk] replacing the volume's densities (its
    gradient flows back); ``pose``: optional tensor (6,) = (t_x, t_y, t_z, w_x, w_y, w_z) of a rigid
    motion of the volume about ``center`` (world; default the volume's centre). Returns
    ``intensity`` and ``photon_prob`` [N, H, W], and with ``area_density`` the per-material area
    densities [N, M, H, W] (g/cm^2, differentiable too). With ``recompute`` the area densities are
    not held from the forward to the backward pass but recomputed there (one more forward pass).

    ``distributed``: the views are this rank's share of a view list sharded over a process group
    (``group``, default the default group; deepdrr_gb300.replicas.shard gives the shares), each rank
    holding its own copy of the volume, and the loss is a sum over all ranks' views. The backward
    then sums the density and pose gradients over the group (one all-reduce of the density
    gradient, one of the six pose numbers), so every rank gets the gradient of the global loss.
    """
    global _PROJECT
    if len(projector.volumes) != 1:
        raise ValueError("differentiable projection supports one volume")
    if projector.attenuate_outside_volume:
        raise ValueError("differentiable projection does not support attenuate_outside_volume")
    if _PROJECT is None:
        _PROJECT = _function()
    cams = projector._prepare_project(camera_projections)
    c = projector.volume_center_world(0) if center is None else center
    state = _State(projector, cams, c, recompute, area_density, distributed, group)
    inten, prob, ad = _PROJECT.apply(density, pose, state)
    out = {"intensity": inten, "photon_prob": prob}
    if area_density:
        out["area_density"] = ad
    return out
