"""Camera and frame geometry at the projector boundary.

DeepDRR takes its geometry from the external ``killeengeo`` package (re-exported by
deepdrr/geo/__init__.py:19-66), which is not vendored in the reference. The projector reads only
three things from a camera projection (deepdrr/projector/projector.py:711, 803, 813):

* ``world_from_index[:-1, :]`` -- a 3x3 matrix W with ray(u, v) = W @ [u, v, 1] the world-space
  vector from the source towards pixel (u, v) (pixel centres at u + 0.5);
* ``center_in_world`` -- the source position;
* ``intrinsic.sensor_size`` / ``sensor_width`` / ``sensor_height``.

This module restates that contract with a pinhole model: ``index_from_world = K [R | t]`` and
``world_from_index = [[R^T K^-1], [0, 0, 0]]`` (a right inverse of the 3x4 projection), so the
ray vector has unit depth along the principal axis. Any object exposing the same three
attributes (for example a killeengeo ``CameraProjection``) is accepted by ``Projector.project``.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np


def _as_vec3(x) -> np.ndarray:
    a = np.asarray(x, dtype=np.float64).reshape(-1)
    if a.shape[0] == 4:
        a = a[:3]
    if a.shape != (3,):
        raise ValueError(f"expected a 3-vector, got shape {np.shape(x)}")
    return a


class FrameTransform:
    """A 4x4 homogeneous rigid (or affine) transform ``B_from_A``."""

    def __init__(self, data=None):
        if data is None:
            data = np.eye(4)
        if isinstance(data, FrameTransform):
            data = data.data
        a = np.array(data, dtype=np.float64)
        if a.shape == (3, 4):
            a = np.vstack([a, [0.0, 0.0, 0.0, 1.0]])
        if a.shape != (4, 4):
            raise ValueError(f"FrameTransform needs a 4x4 or 3x4 matrix, got {a.shape}")
        self.data = a

    @classmethod
    def identity(cls) -> "FrameTransform":
        return cls(np.eye(4))

    @classmethod
    def from_rt(cls, rotation=None, translation=None) -> "FrameTransform":
        m = np.eye(4)
        if rotation is not None:
            m[:3, :3] = np.asarray(rotation, dtype=np.float64)
        if translation is not None:
            m[:3, 3] = _as_vec3(translation)
        return cls(m)

    @classmethod
    def from_scaling(cls, scaling, translation=None) -> "FrameTransform":
        m = np.eye(4)
        m[:3, :3] = np.diag(_as_vec3(np.broadcast_to(np.asarray(scaling, dtype=np.float64), (3,))))
        if translation is not None:
            m[:3, 3] = _as_vec3(translation)
        return cls(m)

    @property
    def R(self) -> np.ndarray:
        return self.data[:3, :3]

    @property
    def t(self) -> np.ndarray:
        return self.data[:3, 3]

    def inverse(self) -> "FrameTransform":
        return FrameTransform(np.linalg.inv(self.data))

    @property
    def inv(self) -> "FrameTransform":
        return self.inverse()

    def toarray(self) -> np.ndarray:
        return self.data.copy()

    def __array__(self, dtype=None, copy=None):
        return self.data.astype(dtype) if dtype is not None else self.data.copy()

    def __matmul__(self, other):
        if isinstance(other, FrameTransform):
            return FrameTransform(self.data @ other.data)
        o = np.asarray(other, dtype=np.float64)
        if o.shape == (3,):  # a point
            return self.data[:3, :3] @ o + self.data[:3, 3]
        if o.shape == (4,):
            return self.data @ o
        raise TypeError(f"cannot apply a FrameTransform to shape {o.shape}")

    def __repr__(self) -> str:
        return f"FrameTransform(\n{self.data}\n)"


def rotation_from_euler(axis: str, angle: float, degrees: bool = False) -> np.ndarray:
    """Rotation matrix about a single axis 'x', 'y' or 'z'."""
    a = np.deg2rad(angle) if degrees else float(angle)
    c, s = np.cos(a), np.sin(a)
    if axis == "x":
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]], dtype=np.float64)
    if axis == "y":
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], dtype=np.float64)
    if axis == "z":
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], dtype=np.float64)
    raise ValueError(f"unknown axis {axis!r}")


def rotation_from_rotvec(rotvec) -> np.ndarray:
    """Rodrigues' formula: rotation by |rotvec| radians about rotvec/|rotvec|."""
    r = _as_vec3(rotvec)
    theta = float(np.linalg.norm(r))
    if theta < 1e-15:
        return np.eye(3)
    k = r / theta
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(theta) * K + (1 - np.cos(theta)) * (K @ K)


class CameraIntrinsicTransform:
    """Pinhole intrinsics K (3x3, pixels) plus the sensor size."""

    def __init__(self, data, sensor_height: int, sensor_width: int):
        self.data = np.array(data, dtype=np.float64).reshape(3, 3)
        self.sensor_height = int(sensor_height)
        self.sensor_width = int(sensor_width)

    @classmethod
    def from_sizes(cls, sensor_size: Tuple[int, int], pixel_size: float,
                   source_to_detector_distance: float) -> "CameraIntrinsicTransform":
        """``sensor_size`` = (width, height); focal length SDD / pixel_size (simple_device.py:66-73)."""
        w, h = int(sensor_size[0]), int(sensor_size[1])
        f = float(source_to_detector_distance) / float(pixel_size)
        K = np.array([[f, 0.0, w / 2.0], [0.0, f, h / 2.0], [0.0, 0.0, 1.0]])
        return cls(K, sensor_height=h, sensor_width=w)

    @property
    def fx(self) -> float:
        return float(self.data[0, 0])

    @property
    def fy(self) -> float:
        return float(self.data[1, 1])

    @property
    def cx(self) -> float:
        return float(self.data[0, 2])

    @property
    def cy(self) -> float:
        return float(self.data[1, 2])

    @property
    def sensor_size(self) -> Tuple[int, int]:
        return (self.sensor_width, self.sensor_height)


class CameraProjection:
    """``index_from_world = K [R | t]`` with ``extrinsic = camera3d_from_world``."""

    def __init__(self, intrinsic: CameraIntrinsicTransform, extrinsic: FrameTransform):
        self.intrinsic = intrinsic
        self.extrinsic = FrameTransform(extrinsic)

    @property
    def camera3d_from_world(self) -> FrameTransform:
        return self.extrinsic

    @property
    def world_from_camera3d(self) -> FrameTransform:
        return self.extrinsic.inverse()

    @property
    def index_from_world(self) -> np.ndarray:
        return self.intrinsic.data @ self.extrinsic.data[:3, :]

    @property
    def world_from_index(self) -> np.ndarray:
        """4x3 right inverse of ``index_from_world``: rows 0-2 map [u, v, 1] to the ray vector."""
        m = np.zeros((4, 3))
        m[:3, :] = self.world_from_camera3d.R @ np.linalg.inv(self.intrinsic.data)
        return m

    @property
    def center_in_world(self) -> np.ndarray:
        return self.world_from_camera3d.t.copy()

    @property
    def sensor_width(self) -> int:
        return self.intrinsic.sensor_width

    @property
    def sensor_height(self) -> int:
        return self.intrinsic.sensor_height

    @classmethod
    def from_view(cls, point, direction, up=(0.0, -1.0, 0.0), *, source_to_detector_distance: float,
                  pixel_size: float, sensor_size: Tuple[int, int],
                  source_to_point_fraction: float = 0.5,
                  source_to_point_distance: Optional[float] = None) -> "CameraProjection":
        """Source on the line through ``point`` along ``direction`` (source -> detector), placed
        ``source_to_point_fraction * SDD`` before ``point``; image up (-v) follows ``up``.
        Mirrors the behaviour of SimpleDevice.set_view (device/simple_device.py:80-165)."""
        p = _as_vec3(point)
        d = _as_vec3(direction)
        d = d / np.linalg.norm(d)
        spd = (source_to_point_distance if source_to_point_distance is not None
               else source_to_detector_distance * source_to_point_fraction)
        src = p - d * spd
        upv = _as_vec3(up)
        y = -(upv - np.dot(upv, d) * d)
        if np.linalg.norm(y) < 1e-9:  # up parallel to the view direction: pick any perpendicular
            alt = np.array([1.0, 0.0, 0.0]) if abs(d[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
            y = -(alt - np.dot(alt, d) * d)
        y = y / np.linalg.norm(y)
        x = np.cross(y, d)
        R = np.stack([x, y, d])  # camera3d_from_world rotation: rows are camera axes in world
        ext = FrameTransform.from_rt(R, -R @ src)
        intr = CameraIntrinsicTransform.from_sizes(sensor_size, pixel_size, source_to_detector_distance)
        return cls(intr, ext)


def view_arrays(proj) -> Tuple[np.ndarray, np.ndarray, int, int]:
    """(world_from_index 3x3 float64, source 3 float64, width, height) of any camera projection
    exposing ``world_from_index``, ``center_in_world`` and a sensor size."""
    W = np.asarray(proj.world_from_index, dtype=np.float64)
    W = W[:3, :3] if W.shape[0] >= 3 else W
    src = _as_vec3(np.asarray(proj.center_in_world, dtype=np.float64))
    if hasattr(proj, "sensor_width"):
        w, h = int(proj.sensor_width), int(proj.sensor_height)
    else:
        w, h = (int(x) for x in proj.intrinsic.sensor_size)
    return W, src, w, h
