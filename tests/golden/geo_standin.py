"""Homogeneous-geometry primitives standing in for killeengeo (TEST INFRASTRUCTURE ONLY).

The reference's device classes (deepdrr/device/{device,simple_device,mobile_carm}.py) compute their
poses with killeengeo, a dependency that is neither vendored with the reference nor installed here.
To run that code as it stands and record its camera poses (tests/golden/make_device_vectors.py),
this module restates the part of killeengeo's published behaviour those classes use: points and
vectors as homogeneous 3-vectors (w = 1 / w = 0), 4x4 frame transforms composed with `@` (a point
takes rotation and translation, a vector rotation only), `from_rt` with a rotation matrix or a
scipy Rotation, `inverse`, and the pinhole intrinsics of `CameraIntrinsicTransform.from_sizes`
(f = source-to-detector distance / pixel size, principal point at the sensor centre).

Two conventions are this module's own reading of killeengeo and are stated here: `angle` is the
arccos of the normalised dot product clipped to [-1, 1], and `hat` divides by the Euclidean norm.
The golden vectors therefore pin the reference's frame composition (which transforms, in which
order, about which points), not killeengeo's arithmetic itself.
"""
from __future__ import annotations

import numpy as np
from scipy.spatial.transform import Rotation

__all__ = ["Point", "Vector", "Point3D", "Vector3D", "point", "vector", "FrameTransform", "F", "frame_transform",
           "CameraIntrinsicTransform", "CameraProjection", "Transform", "get_data", "Rotation"]


def get_data(x) -> np.ndarray:
    if isinstance(x, (Point, Vector)):
        return x.data.copy()
    if isinstance(x, FrameTransform):
        return x.data.copy()
    return np.asarray(x, dtype=np.float64)


class _PV:
    def __init__(self, data):
        self.data = np.asarray(data, dtype=np.float64).reshape(3).copy()

    def __array__(self, dtype=None, copy=None):
        return self.data.astype(dtype) if dtype is not None else self.data.copy()

    def __getitem__(self, i):
        return self.data[i]

    def __iter__(self):
        return iter(self.data.tolist())

    def __len__(self):
        return 3


class Vector(_PV):
    def __add__(self, o):
        if isinstance(o, Point):
            return Point(self.data + o.data)
        return Vector(self.data + get_data(o))

    __radd__ = __add__

    def __sub__(self, o):
        return Vector(self.data - get_data(o))

    def __neg__(self):
        return Vector(-self.data)

    def __mul__(self, s):
        return Vector(self.data * float(s))

    __rmul__ = __mul__

    def __truediv__(self, s):
        return Vector(self.data / float(s))

    def norm(self) -> float:
        return float(np.linalg.norm(self.data))

    def hat(self) -> "Vector":
        return Vector(self.data / np.linalg.norm(self.data))

    def dot(self, o) -> float:
        return float(np.dot(self.data, get_data(o)))

    def cross(self, o) -> "Vector":
        return Vector(np.cross(self.data, get_data(o)))

    def angle(self, o) -> float:
        b = get_data(o)
        c = np.dot(self.data, b) / (np.linalg.norm(self.data) * np.linalg.norm(b))
        return float(np.arccos(np.clip(c, -1.0, 1.0)))


class Point(_PV):
    def __add__(self, o):
        return Point(self.data + get_data(o))

    def __sub__(self, o):
        if isinstance(o, Point):
            return Vector(self.data - o.data)
        return Point(self.data - get_data(o))


Point3D, Vector3D = Point, Vector


def point(*args) -> Point:
    if len(args) == 1:
        return Point(get_data(args[0]))
    return Point(np.array(args, dtype=np.float64))


def vector(*args) -> Vector:
    if len(args) == 1:
        return Vector(get_data(args[0]))
    return Vector(np.array(args, dtype=np.float64))


class FrameTransform:
    def __init__(self, data=None):
        self.data = np.eye(4) if data is None else np.asarray(data, dtype=np.float64).reshape(4, 4).copy()

    @classmethod
    def identity(cls):
        return cls()

    @classmethod
    def from_rt(cls, rotation=None, translation=None):
        T = np.eye(4)
        if rotation is not None:
            T[:3, :3] = rotation.as_matrix() if isinstance(rotation, Rotation) else np.asarray(rotation, np.float64)
        if translation is not None:
            T[:3, 3] = get_data(translation)
        return cls(T)

    @classmethod
    def from_translation(cls, translation):
        return cls.from_rt(translation=translation)

    def inverse(self):
        return FrameTransform(np.linalg.inv(self.data))

    @property
    def inv(self):
        return self.inverse()

    def __matmul__(self, o):
        if isinstance(o, FrameTransform):
            return FrameTransform(self.data @ o.data)
        if isinstance(o, Vector):
            return Vector(self.data[:3, :3] @ o.data)
        if isinstance(o, Point):
            return Point(self.data[:3, :3] @ o.data + self.data[:3, 3])
        raise TypeError(f"cannot apply a frame transform to {type(o)}")

    def __array__(self, dtype=None, copy=None):
        return self.data.astype(dtype) if dtype is not None else self.data.copy()


F = FrameTransform
Transform = FrameTransform


def frame_transform(x=None) -> FrameTransform:
    if x is None:
        return FrameTransform()
    if isinstance(x, FrameTransform):
        return x
    if isinstance(x, Rotation):
        return FrameTransform.from_rt(rotation=x)
    a = np.asarray(x, dtype=np.float64)
    if a.shape == (3, 3):
        return FrameTransform.from_rt(rotation=a)
    return FrameTransform(a)


class CameraIntrinsicTransform:
    def __init__(self, data, sensor_height: int, sensor_width: int):
        self.data = np.asarray(data, dtype=np.float64).reshape(3, 3).copy()
        self.sensor_height = int(sensor_height)
        self.sensor_width = int(sensor_width)

    @classmethod
    def from_sizes(cls, sensor_size, pixel_size, source_to_detector_distance):
        w, h = (sensor_size, sensor_size) if np.isscalar(sensor_size) else sensor_size
        f = float(source_to_detector_distance) / float(pixel_size)
        return cls([[f, 0.0, w / 2.0], [0.0, f, h / 2.0], [0.0, 0.0, 1.0]], sensor_height=h, sensor_width=w)


class CameraProjection:
    def __init__(self, intrinsic, extrinsic):
        self.intrinsic = intrinsic
        self.extrinsic = frame_transform(extrinsic)
