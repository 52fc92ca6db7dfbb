"""X-ray devices: the objects that set the projector's view in ``Projector(volume, device=...)``.

Restates the reference's device classes (deepdrr/device/device.py, simple_device.py,
mobile_carm.py, camera_projection_device.py) on this package's geometry (``geo``), since the
reference builds them on killeengeo, which is not vendored. A device owns a pose and produces a
``CameraProjection`` (``get_camera_projection``); the projector also reads its
``source_to_detector_distance``, ``camera_intrinsics`` and detector size (projector.py:641-650).

Frames: ``device`` (the device's base, placed in the world by ``world_from_device``) and
``camera3d`` (origin at the X-ray source, +z along the principal ray towards the detector, image
u along +x and v along +y). Lengths in millimetres.
"""
from __future__ import annotations

import math
from typing import List, Optional, Sequence, Tuple

import numpy as np
from scipy.spatial.transform import Rotation

from .geo import CameraIntrinsicTransform, CameraProjection, FrameTransform

__all__ = ["Device", "SimpleDevice", "MobileCArm", "CameraProjectionDevice", "pose_vector_angles"]


def _vec(x) -> np.ndarray:
    a = np.asarray(x, dtype=np.float64).reshape(-1)
    return a[:3]


def _apply_point(T: FrameTransform, p) -> np.ndarray:
    return T.data[:3, :3] @ _vec(p) + T.data[:3, 3]


def _apply_vector(T: FrameTransform, v) -> np.ndarray:
    return T.data[:3, :3] @ _vec(v)


def _angle(a, b) -> float:
    a, b = _vec(a), _vec(b)
    c = float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)))
    return math.acos(max(-1.0, min(1.0, c)))


def _radians(x: float, degrees: bool) -> float:
    return math.radians(x) if degrees else float(x)


def _rotation_frame(rotvec, translation=None) -> FrameTransform:
    return FrameTransform.from_rt(Rotation.from_rotvec(_vec(rotvec)).as_matrix(), translation)


class Device:
    """Base class (device/device.py:7-209): subclasses provide ``device_from_camera3d`` and set
    ``sensor_height``, ``sensor_width``, ``pixel_size``, ``source_to_detector_distance``,
    ``camera_intrinsics`` and ``world_from_device``."""

    sensor_height: int
    sensor_width: int
    pixel_size: float
    source_to_detector_distance: float
    world_from_device: FrameTransform

    @property
    def detector_height(self) -> float:
        """Detector height in mm."""
        return self.sensor_height * self.pixel_size

    @property
    def detector_width(self) -> float:
        """Detector width in mm."""
        return self.sensor_width * self.pixel_size

    @property
    def device_from_world(self) -> FrameTransform:
        return self.world_from_device.inverse()

    @property
    def device_from_camera3d(self) -> FrameTransform:
        raise NotImplementedError

    @property
    def camera3d_from_device(self) -> FrameTransform:
        return self.device_from_camera3d.inverse()

    @property
    def world_from_camera3d(self) -> FrameTransform:
        return self.world_from_device @ self.device_from_camera3d

    @property
    def camera3d_from_world(self) -> FrameTransform:
        return self.camera3d_from_device @ self.device_from_world

    def get_camera_projection(self) -> CameraProjection:
        """The index_from_world camera projection of the current pose."""
        return CameraProjection(self.camera_intrinsics, self.camera3d_from_world)

    @property
    def index_from_world(self) -> CameraProjection:
        return self.get_camera_projection()

    @property
    def world_from_index(self) -> np.ndarray:
        return self.get_camera_projection().world_from_index

    @property
    def principle_ray(self) -> np.ndarray:
        """Unit principal ray (source -> detector) in the device frame."""
        v = _apply_vector(self.device_from_camera3d, [0.0, 0.0, 1.0])
        return v / np.linalg.norm(v)

    @property
    def principle_ray_in_world(self) -> np.ndarray:
        v = _apply_vector(self.world_from_device, self.principle_ray)
        return v / np.linalg.norm(v)

    @property
    def source_in_world(self) -> np.ndarray:
        return _apply_point(self.world_from_camera3d, [0.0, 0.0, 0.0])

    def get_frustum_points(self) -> List[np.ndarray]:
        """World points of the source, the detector centre and the detector corners."""
        sdd = self.source_to_detector_distance
        cx = self.pixel_size * self.sensor_height / 2.0
        cy = self.pixel_size * self.sensor_width / 2.0
        pts = [[0.0, 0.0, 0.0], [0.0, 0.0, sdd], [-cx, cy, sdd], [cx, cy, sdd], [-cx, -cy, sdd], [cx, -cy, sdd]]
        return [_apply_point(self.world_from_camera3d, p) for p in pts]


class SimpleDevice(Device):
    """A C-arm positioned by a point, a direction and an up vector (device/simple_device.py:10-178).

    The point is the one placed ``source_to_point_distance`` (default ``source_to_point_fraction``
    of the SDD) from the source along the principal ray; the up vector's projection onto the image
    plane becomes the image's -v direction."""

    def __init__(self, sensor_height: int = 384, sensor_width: int = 384, pixel_size: float = 1.0,
                 source_to_detector_distance: float = 1000.0, world_from_device: Optional[FrameTransform] = None):
        self.sensor_height = int(sensor_height)
        self.sensor_width = int(sensor_width)
        self.pixel_size = float(pixel_size)
        self.source_to_detector_distance = float(source_to_detector_distance)
        self.world_from_device = FrameTransform(world_from_device)
        self._device_from_camera3d = FrameTransform.identity()
        self.set_view([0, 0, 0], [0, 0, 1], [0, -1, 0])

    def scale_sensor(self, detector_size: float) -> None:
        """Set the pixel size so that the shorter side of the sensor spans ``detector_size`` mm."""
        self.pixel_size = detector_size / min(self.sensor_height, self.sensor_width)

    @property
    def camera_intrinsics(self) -> CameraIntrinsicTransform:
        f = self.source_to_detector_distance / self.pixel_size
        K = np.array([[f, 0.0, self.sensor_width / 2.0], [0.0, f, self.sensor_height / 2.0], [0.0, 0.0, 1.0]])
        return CameraIntrinsicTransform(K, sensor_height=self.sensor_height, sensor_width=self.sensor_width)

    def set_view(self, point=None, direction=None, up=None, source_to_point_distance: Optional[float] = None,
                 source_to_point_fraction: float = 0.5) -> None:
        """Point the device (simple_device.py:80-165). ``point`` None keeps the current point,
        ``direction`` None keeps the current principal ray, ``up`` None means the device's -y."""
        if source_to_point_distance is None:
            source_to_point_distance = self.source_to_detector_distance * source_to_point_fraction
        if point is None:
            point_d = _apply_point(self._device_from_camera3d, [0.0, 0.0, source_to_point_distance])
        else:
            point_d = _apply_point(self.device_from_world, point)
        if direction is None:
            dir_d = _apply_vector(self._device_from_camera3d, [0.0, 0.0, 1.0])
        else:
            dir_d = _apply_vector(self.device_from_world, direction)
        up_d = np.array([0.0, -1.0, 0.0]) if up is None else _apply_vector(self.device_from_world, up)

        # "ray" frame: origin at the point, z along the direction (the rotation turning z onto it)
        z = np.array([0.0, 0.0, 1.0])
        axis = np.cross(z, dir_d)
        if np.linalg.norm(axis) < 1e-6:
            rotvec = np.array([math.pi, 0.0, 0.0]) if np.dot(z, dir_d) < 0 else np.zeros(3)
        else:
            rotvec = axis / np.linalg.norm(axis) * _angle(z, dir_d)
        device_from_ray = _rotation_frame(rotvec, point_d)
        # turn about z so that the up vector's projection onto the image plane is -y
        neg_y = np.array([0.0, -1.0, 0.0])
        up_r = _apply_vector(device_from_ray.inverse(), up_d)
        up_plane = np.array([up_r[0], up_r[1], 0.0])
        axis = np.cross(neg_y, up_plane)
        if np.linalg.norm(axis) < 1e-6:
            rotvec = np.zeros(3)
        else:
            rotvec = axis / np.linalg.norm(axis) * _angle(neg_y, up_plane)
        ray_from_ray_up = _rotation_frame(rotvec)
        ray_up_from_camera3d = FrameTransform.from_rt(translation=[0.0, 0.0, -source_to_point_distance])
        self._device_from_camera3d = device_from_ray @ ray_from_ray_up @ ray_up_from_camera3d

    @property
    def device_from_camera3d(self) -> FrameTransform:
        return self._device_from_camera3d

    def __str__(self) -> str:
        return (f"SimpleDevice(sensor_height={self.sensor_height}, sensor_width={self.sensor_width}, "
                f"pixel_size={self.pixel_size}, source_to_detector_distance={self.source_to_detector_distance})")


def pose_vector_angles(pose) -> Tuple[float, float]:
    """C-arm angles (alpha, beta) in radians whose principal ray is ``pose`` (mobile_carm.py:20-34)."""
    x, y, z = (float(c) for c in _vec(pose))
    return -math.atan2(y, math.sqrt(x * x + z * z)), math.atan2(x, z)


class MobileCArm(Device):
    """A mobile C-arm with orbital (alpha), angulation (beta) and detector (gamma) rotations about
    an isocenter that translates in the device frame (device/mobile_carm.py:37-541). Defaults
    follow the reference (a Siemens Cios-like geometry: SDD 1020 mm, source 530 mm below the
    isocenter, 1536^2 sensor at 0.194 mm)."""

    def __init__(self, world_from_device: Optional[FrameTransform] = None, isocenter=(0.0, 0.0, 0.0),
                 alpha: float = 0.0, beta: float = 0.0, gamma: float = 0.0, degrees: bool = True,
                 horizontal_movement: float = 200.0, vertical_travel: float = 430.0,
                 min_alpha: float = -40.0, max_alpha: float = 110.0, min_beta: float = -225.0, max_beta: float = 225.0,
                 source_to_detector_distance: float = 1020.0, source_to_isocenter_vertical_distance: float = 530.0,
                 source_to_isocenter_horizontal_offset: float = 0.0, immersion_depth: float = 730.0,
                 free_space: float = 820.0, sensor_height: int = 1536, sensor_width: int = 1536,
                 pixel_size: float = 0.194, rotate_camera_left: bool = True, enforce_isocenter_bounds: bool = False):
        self.world_from_device = FrameTransform(world_from_device)
        self.enforce_isocenter_bounds = enforce_isocenter_bounds
        self.isocenter = _vec(isocenter).copy()
        self.alpha = _radians(alpha, degrees)
        self.beta = _radians(beta, degrees)
        self.gamma = _radians(gamma, degrees)
        self.horizontal_movement = float(horizontal_movement)
        self.vertical_travel = float(vertical_travel)
        self.min_alpha = _radians(min_alpha, degrees)
        self.max_alpha = _radians(max_alpha, degrees)
        self.min_beta = _radians(min_beta, degrees)
        self.max_beta = _radians(max_beta, degrees)
        self.source_to_detector_distance = float(source_to_detector_distance)
        self.source_to_isocenter_vertical_distance = float(source_to_isocenter_vertical_distance)
        self.source_to_isocenter_horizontal_offset = float(source_to_isocenter_horizontal_offset)
        self.immersion_depth = float(immersion_depth)
        self.free_space = float(free_space)
        self.pixel_size = float(pixel_size)
        self.sensor_width = int(sensor_width)
        self.sensor_height = int(sensor_height)
        self.camera_intrinsics = CameraIntrinsicTransform.from_sizes(
            (self.sensor_width, self.sensor_height), self.pixel_size, self.source_to_detector_distance)
        self.rotate_camera_left = rotate_camera_left
        if enforce_isocenter_bounds and (np.any(self.isocenter < self.min_isocenter)
                                         or np.any(self.isocenter > self.max_isocenter)):
            raise ValueError(f"isocenter {self.isocenter} is out of bounds; position the C-arm in the world "
                             f"with world_from_device")
        self.viewpoint_in_arm = np.array([0.0, self.source_to_isocenter_horizontal_offset, 0.0])
        self._enforce_bounds()

    def __str__(self) -> str:
        return (f"MobileCArm(isocenter={np.array_str(self.isocenter)}, alpha={math.degrees(self.alpha)}, "
                f"beta={math.degrees(self.beta)}, degrees=True)")

    def to_config(self) -> dict:
        """JSON-safe keyword arguments that rebuild this C-arm in its current pose."""
        return dict(world_from_device=self.world_from_device.data.tolist(), isocenter=self.isocenter.tolist(),
                    alpha=self.alpha, beta=self.beta, gamma=self.gamma, degrees=False,
                    horizontal_movement=self.horizontal_movement, vertical_travel=self.vertical_travel,
                    min_alpha=self.min_alpha, max_alpha=self.max_alpha, min_beta=self.min_beta,
                    max_beta=self.max_beta, source_to_detector_distance=self.source_to_detector_distance,
                    source_to_isocenter_vertical_distance=self.source_to_isocenter_vertical_distance,
                    source_to_isocenter_horizontal_offset=self.source_to_isocenter_horizontal_offset,
                    immersion_depth=self.immersion_depth, free_space=self.free_space,
                    sensor_height=self.sensor_height, sensor_width=self.sensor_width, pixel_size=self.pixel_size,
                    rotate_camera_left=self.rotate_camera_left,
                    enforce_isocenter_bounds=self.enforce_isocenter_bounds)

    @property
    def max_isocenter(self) -> np.ndarray:
        return np.array([self.horizontal_movement, self.horizontal_movement, self.vertical_travel]) / 2

    @property
    def min_isocenter(self) -> np.ndarray:
        return -self.max_isocenter

    @property
    def isocenter_in_world(self) -> np.ndarray:
        return _apply_point(self.world_from_device, self.isocenter)

    @property
    def device_from_arm(self) -> FrameTransform:
        """Rotate by alpha about x, then by beta about y (fixed axes), then move to the isocenter."""
        R = Rotation.from_euler("xy", [self.alpha, self.beta]).as_matrix()
        return FrameTransform.from_rt(R, self.isocenter)

    @property
    def arm_from_device(self) -> FrameTransform:
        return self.device_from_arm.inverse()

    @property
    def camera3d_from_device(self) -> FrameTransform:
        camera3d_from_arm = FrameTransform.from_rt(
            translation=[0.0, -self.source_to_isocenter_horizontal_offset, self.source_to_isocenter_vertical_distance])
        if self.rotate_camera_left:
            camera3d_from_arm = FrameTransform.from_rt(
                Rotation.from_euler("z", 90, degrees=True).as_matrix()) @ camera3d_from_arm
        gamma_rotation = FrameTransform.from_rt(Rotation.from_euler("z", self.gamma).as_matrix())
        return gamma_rotation @ camera3d_from_arm @ self.arm_from_device

    @property
    def device_from_camera3d(self) -> FrameTransform:
        return self.camera3d_from_device.inverse()

    def get_camera3d_from_world(self) -> FrameTransform:
        return self.camera3d_from_device @ self.device_from_world

    @property
    def camera3d_from_world(self) -> FrameTransform:
        return self.get_camera3d_from_world()

    def get_camera_projection(self) -> CameraProjection:
        return CameraProjection(self.camera_intrinsics, self.get_camera3d_from_world())

    @property
    def viewpoint(self) -> np.ndarray:
        """The point on the principal ray where the object of interest belongs (device frame)."""
        return _apply_point(self.device_from_arm, self.viewpoint_in_arm)

    @property
    def viewpoint_in_world(self) -> np.ndarray:
        return _apply_point(self.world_from_device, self.viewpoint)

    @property
    def principle_ray(self) -> np.ndarray:
        v = _apply_vector(self.device_from_arm, [0.0, 0.0, 1.0])
        return v / np.linalg.norm(v)

    @property
    def source_in_arm(self) -> np.ndarray:
        return np.array([0.0, self.source_to_isocenter_horizontal_offset, -self.source_to_isocenter_vertical_distance])

    @property
    def source_in_device(self) -> np.ndarray:
        return _apply_point(self.device_from_arm, self.source_in_arm)

    def _enforce_bounds(self) -> None:
        if self.enforce_isocenter_bounds:
            self.isocenter = np.clip(self.isocenter, self.min_isocenter, self.max_isocenter)
        self.alpha = float(np.clip(self.alpha, self.min_alpha, self.max_alpha))
        self.beta = float(np.clip(self.beta, self.min_beta, self.max_beta))

    def move_by(self, delta_isocenter=None, delta_alpha: Optional[float] = None, delta_beta: Optional[float] = None,
                delta_gamma: Optional[float] = None, degrees: bool = True) -> None:
        """Move relative to the current pose (isocenter change in device coordinates)."""
        if delta_isocenter is not None:
            self.isocenter = self.isocenter + _vec(delta_isocenter)
        for name, d in (("alpha", delta_alpha), ("beta", delta_beta), ("gamma", delta_gamma)):
            if d is not None:
                if not np.isscalar(d):
                    raise TypeError(f"delta_{name} must be a scalar")
                setattr(self, name, getattr(self, name) + _radians(float(d), degrees))
        self._enforce_bounds()

    def move_to(self, isocenter=None, isocenter_in_world=None, alpha: Optional[float] = None,
                beta: Optional[float] = None, gamma: Optional[float] = None, degrees: bool = True,
                interest_point_in_world=None, principle_ray_in_world=None) -> None:
        """Move to an absolute pose (mobile_carm.py:349-413). ``principle_ray_in_world`` overrides
        alpha and beta; ``interest_point_in_world`` moves the isocenter so the point keeps its
        place along the principal ray; ``isocenter_in_world`` overrides ``isocenter``."""
        old_ray = self.principle_ray
        if principle_ray_in_world is not None:
            alpha, beta = pose_vector_angles(_apply_vector(self.device_from_world, principle_ray_in_world))
            if gamma is not None:
                gamma = _radians(float(gamma), degrees)
            degrees = False
        if alpha is not None:
            self.alpha = _radians(float(alpha), degrees)
        if beta is not None:
            self.beta = _radians(float(beta), degrees)
        if gamma is not None:
            self.gamma = _radians(float(gamma), degrees)
        if interest_point_in_world is not None:
            ray = self.principle_ray
            ip = _apply_point(self.device_from_world, interest_point_in_world)
            isocenter = ip - float(np.dot(ip - self.isocenter, old_ray / np.linalg.norm(old_ray))) * ray
        elif isocenter_in_world is not None:
            isocenter = _apply_point(self.device_from_world, isocenter_in_world)
        if isocenter is not None:
            self.isocenter = _vec(isocenter).copy()
        self._enforce_bounds()

    def reposition(self, viewpoint_in_world=None, device_in_world=None) -> None:
        """Reset the pose to zero and place the device so its viewpoint (or origin) is at the given
        world point (mobile_carm.py:415-436)."""
        self.move_to(isocenter=[0.0, 0.0, 0.0], alpha=0.0, beta=0.0, degrees=False)
        if device_in_world is None:
            if viewpoint_in_world is None:
                raise ValueError("reposition needs viewpoint_in_world or device_in_world")
            device_in_world = _vec(viewpoint_in_world) - self.viewpoint_in_arm
        self.world_from_device = FrameTransform.from_rt(translation=device_in_world)


class CameraProjectionDevice(Device):
    """A fixed camera projection presented as a device (device/camera_projection_device.py:10-50)."""

    def __init__(self, projection: CameraProjection, pixel_size: float = 1.0):
        self.pixel_size = float(pixel_size)
        self.projection = projection

    @property
    def projection(self) -> CameraProjection:
        return self._projection

    @projection.setter
    def projection(self, projection: CameraProjection) -> None:
        self._projection = projection
        self.sensor_height = projection.intrinsic.sensor_height
        self.sensor_width = projection.intrinsic.sensor_width
        self.camera_intrinsics = projection.intrinsic
        self.source_to_detector_distance = projection.intrinsic.fx * self.pixel_size
        self.world_from_device = projection.world_from_camera3d

    @property
    def device_from_camera3d(self) -> FrameTransform:
        return FrameTransform.identity()
