"""deepdrr_gb300: a GB300-native (sm_103a) DeepDRR volume projector.

``Projector`` is a drop-in for ``deepdrr.Projector`` on the volume path: ray march through one or
more CT volumes with trilinear sampling and material fractions, per-material path lengths, and
polychromatic Beer-Lambert attenuation with optional neglog, all in hand-written CUDA kernels
reached through the C ABI of ``libdrr_gb300.so`` (``include/drr_gb300.h``).
"""
from . import geo, tables
from .device import CameraProjectionDevice, Device, MobileCArm, SimpleDevice
from .geo import CameraIntrinsicTransform, CameraProjection, FrameTransform
from .mesh import Mesh
from .projector import DeprecationError, Projector
from .volume import Volume, format_materials, hu_to_density, segment_thresholds

__version__ = "0.1.0"

__all__ = [
    "Projector", "Volume", "CameraIntrinsicTransform", "CameraProjection", "FrameTransform",
    "DeprecationError", "geo", "tables", "Mesh", "Device", "SimpleDevice", "MobileCArm", "CameraProjectionDevice", "hu_to_density", "segment_thresholds", "format_materials",
]
