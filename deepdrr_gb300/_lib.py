"""ctypes binding of ``libdrr_gb300.so`` (the C ABI declared in ``include/drr_gb300.h``).

The shared library is built in-tree by ``deepdrr_gb300.build``. Loading fails loudly when it is
missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

from . import build as _build

DRR_OK = 0
DRR_ERR_INVALID_ARGUMENT = 1
DRR_ERR_UNSUPPORTED = 2
DRR_ERR_CUDA = 3
DRR_ERR_OUT_OF_MEMORY = 4

DRR_DENSITY_F32 = 0
DRR_DENSITY_F16 = 1
DRR_DENSITY_BF16 = 2

DRR_HU_F32 = 0
DRR_HU_I16 = 1
DRR_HU_F64 = 2

DRR_MAX_VOLUMES = 4
DRR_MAX_MESH_LAYERS = 4
DRR_MESH_ADDITIVE = 1
DRR_MESH_SUBTRACTIVE = 2
DRR_MAX_MATERIALS = 16

DRR_FLAG_ATTENUATE_OUTSIDE = 1 << 0
DRR_FLAG_FULL_MARCH = 1 << 1
DRR_FLAG_PERSISTENT = 1 << 2

# Every symbol the header declares; the CPU test suite checks that the library exports all of them.
EXPORTED_SYMBOLS = (
    "drr_volset_create", "drr_volset_destroy", "drr_volset_set_density", "drr_ingest_hu", "drr_tables_create", "drr_tables_destroy",
    "drr_project", "drr_project_adjoint", "drr_graph_create", "drr_graph_set_views", "drr_graph_launch", "drr_graph_destroy",
    "drr_autotune", "drr_mesh_hits", "drr_mesh_area_density", "drr_add_noise", "drr_poisson_sample", "drr_neglog", "drr_neglog_noalloc", "drr_collected_energy", "drr_clip_upper", "drr_last_error", "drr_version",
)


class DrrError(RuntimeError):
    """A non-OK status returned by libdrr_gb300."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class drr_volume_desc(ctypes.Structure):
    _fields_ = [
        ("density", ctypes.c_void_p),
        ("labels", ctypes.c_void_p),
        ("ni", ctypes.c_int32), ("nj", ctypes.c_int32), ("nk", ctypes.c_int32),
        ("density_type", ctypes.c_int32),
    ]


class _Sized(ctypes.Structure):
    """An argument struct whose first field, struct_size, must hold its own size (the library
    rejects any other value); instances are created with it filled in."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        if "struct_size" not in kwargs:
            self.struct_size = ctypes.sizeof(self)


class drr_project_args(_Sized):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("width", ctypes.c_int32), ("height", ctypes.c_int32),
        ("step", ctypes.c_float), ("max_ray_length", ctypes.c_float),
        ("air_index", ctypes.c_int32), ("flags", ctypes.c_uint32),
        ("n_views", ctypes.c_int32),
        ("priority", ctypes.c_void_p), ("enabled", ctypes.c_void_p),
        ("world_from_index", ctypes.c_void_p), ("source_world", ctypes.c_void_p),
        ("ijk_from_world", ctypes.c_void_p),
        ("intensity", ctypes.c_void_p), ("photon_prob", ctypes.c_void_p),
        ("area_density", ctypes.c_void_p), ("solid_angle", ctypes.c_void_p),
        ("tile_warps_x", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32), ("items_per_grab", ctypes.c_int32),
        ("mesh_area_density", ctypes.c_void_p), ("n_mesh_slots", ctypes.c_int32), ("mesh_material", ctypes.c_void_p),
        ("mesh_hit_alpha", ctypes.c_void_p), ("mesh_hit_facing", ctypes.c_void_p),
        ("mesh_hit_layers", ctypes.c_int32), ("max_mesh_hits", ctypes.c_int32),
    ]


class drr_mesh_desc(ctypes.Structure):
    _fields_ = [
        ("triangles", ctypes.c_void_p), ("slot", ctypes.c_void_p), ("density", ctypes.c_void_p),
        ("layer", ctypes.c_void_p), ("mode", ctypes.c_void_p),
        ("n_triangles", ctypes.c_int32), ("n_slots", ctypes.c_int32), ("n_layers", ctypes.c_int32),
    ]


class drr_adjoint_args(_Sized):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("area_density", ctypes.c_void_p), ("grad_intensity", ctypes.c_void_p),
        ("grad_photon_prob", ctypes.c_void_p), ("grad_area_density", ctypes.c_void_p),
        ("grad_density", ctypes.c_void_p), ("grad_pose", ctypes.c_void_p),
        ("center", ctypes.c_double * 3),
    ]


class drr_tune_result(ctypes.Structure):
    _fields_ = [
        ("tile_warps_x", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32), ("items_per_grab", ctypes.c_int32),
        ("ms_per_view", ctypes.c_float),
    ]


_LIB = None


def library_path() -> Path:
    return _build.BUILD / _build.LIB_NAME


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the library, building it first if it is absent and a toolkit is present."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists() or os.environ.get("DEEPDRR_GB300_REBUILD") == "1":
        if not build_if_missing:
            raise RuntimeError(f"libdrr_gb300.so not found at {path}; run deepdrr_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(str(path))
    vp, i32, st = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int
    lib.drr_volset_create.argtypes = [ctypes.POINTER(drr_volume_desc), i32, i32, vp, ctypes.POINTER(vp)]
    lib.drr_volset_create.restype = st
    lib.drr_volset_destroy.argtypes = [vp]
    lib.drr_volset_destroy.restype = st
    lib.drr_volset_set_density.argtypes = [vp, i32, vp, vp]
    lib.drr_volset_set_density.restype = st
    lib.drr_ingest_hu.argtypes = [vp, i32, i32, i32, i32, ctypes.POINTER(ctypes.c_uint8), vp, i32, vp, vp]
    lib.drr_ingest_hu.restype = st
    lib.drr_tables_create.argtypes = [vp, vp, vp, i32, i32, vp, ctypes.POINTER(vp)]
    lib.drr_tables_create.restype = st
    lib.drr_tables_destroy.argtypes = [vp]
    lib.drr_tables_destroy.restype = st
    lib.drr_project.argtypes = [vp, vp, ctypes.POINTER(drr_project_args), vp]
    lib.drr_project.restype = st
    lib.drr_project_adjoint.argtypes = [vp, vp, ctypes.POINTER(drr_project_args), ctypes.POINTER(drr_adjoint_args), vp]
    lib.drr_project_adjoint.restype = st
    lib.drr_graph_create.argtypes = [vp, vp, ctypes.POINTER(drr_project_args), ctypes.POINTER(vp)]
    lib.drr_graph_create.restype = st
    lib.drr_graph_set_views.argtypes = [vp, vp, vp, vp]
    lib.drr_graph_set_views.restype = st
    lib.drr_graph_launch.argtypes = [vp, vp]
    lib.drr_graph_launch.restype = st
    lib.drr_graph_destroy.argtypes = [vp]
    lib.drr_graph_destroy.restype = st
    lib.drr_autotune.argtypes = [vp, vp, ctypes.POINTER(drr_project_args), i32, vp, ctypes.POINTER(drr_tune_result)]
    lib.drr_autotune.restype = st
    lib.drr_mesh_hits.argtypes = [ctypes.POINTER(drr_mesh_desc), i32, i32, vp, vp, i32, vp, vp, vp]
    lib.drr_mesh_hits.restype = st
    lib.drr_mesh_area_density.argtypes = [ctypes.POINTER(drr_mesh_desc), i32, i32, i32, vp, vp, vp, vp, i32, vp, vp]
    lib.drr_mesh_area_density.restype = st
    lib.drr_add_noise.argtypes = [vp, vp, vp, i32, i32, i32, ctypes.c_double, ctypes.c_uint64, vp]
    lib.drr_add_noise.restype = st
    lib.drr_poisson_sample.argtypes = [vp, ctypes.c_int64, ctypes.c_uint64, vp, vp]
    lib.drr_poisson_sample.restype = st
    lib.drr_neglog.argtypes = [vp, i32, ctypes.c_int64, ctypes.c_float, vp]
    lib.drr_neglog.restype = st
    lib.drr_neglog_noalloc.argtypes = [vp, i32, ctypes.c_int64, ctypes.c_float, vp]
    lib.drr_neglog_noalloc.restype = st
    lib.drr_collected_energy.argtypes = [vp, vp, vp, i32, ctypes.c_int64, ctypes.c_double, vp, vp]
    lib.drr_collected_energy.restype = st
    lib.drr_clip_upper.argtypes = [vp, ctypes.c_int64, ctypes.c_float, vp]
    lib.drr_clip_upper.restype = st
    lib.drr_last_error.argtypes = []
    lib.drr_last_error.restype = ctypes.c_char_p
    lib.drr_version.argtypes = []
    lib.drr_version.restype = ctypes.c_char_p
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != DRR_OK:
        msg = load().drr_last_error().decode("utf-8", "replace")
        raise DrrError(status, msg)
