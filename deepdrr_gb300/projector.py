"""``Projector``: the drop-in replacement of deepdrr.Projector for volume rendering.

Mirrors deepdrr/projector/projector.py (deepdrr v1.2.2): the constructor signature and checks
(projector.py:398-587), ``initialize`` / ``free`` / context manager (:1395-1771), ``project`` /
``__call__`` (:655-707, :1773) with its return types (numpy float32 [H, W] for one view, [N, H, W]
otherwise), and the post-processing order noise -> clip -> neglog (:691-702).

Everything that touches the GPU goes through ``libdrr_gb300.so`` (hand-written sm_103a kernels
behind a C ABI); PyTorch only provides device memory and the current CUDA stream. There is no
CPU fallback: without a CUDA device ``initialize`` raises.

Meshes are rasterised in CUDA (``drr_mesh_*``) instead of the reference's OpenGL depth peeling.
Not carried over: scatter (deprecated in the reference, raises) and ``mode`` (stored but unused by
the reference as well).
"""
from __future__ import annotations

import ctypes
import logging
import math
import warnings
from pathlib import Path
from typing import List, Optional, Sequence, Union

import numpy as np

from . import _lib, geo
from .tables import TableSource, build_tables, configured_source
from .mesh import Mesh
from .volume import Volume

log = logging.getLogger(__name__)


class DeprecationError(Exception):
    """Raised for deprecated features, like the reference (pyvista.DeprecationError)."""


def _listify(x) -> list:
    return list(x) if isinstance(x, (list, tuple)) else [x]


class Projector:
    def __init__(
        self,
        volume: Union[Volume, List[Volume]],
        priorities: Optional[List[int]] = None,
        camera_intrinsics: Optional[geo.CameraIntrinsicTransform] = None,
        device=None,
        step: float = 0.1,
        mode: str = "linear",
        spectrum: Union[np.ndarray, str] = "90KV_AL40",
        add_scatter: Optional[bool] = None,
        scatter_num: int = 0,
        add_noise: bool = False,
        photon_count: int = 10000,
        threads: int = 8,
        max_block_index: int = 65535,
        collected_energy: bool = False,
        neglog: bool = True,
        intensity_upper_bound: Optional[float] = None,
        attenuate_outside_volume: bool = False,
        source_to_detector_distance: float = -1,
        carm=None,
        max_mesh_hits: int = 32,
        mesh_layers: int = 2,
        cuda_device_id: Optional[int] = None,
        *,
        density_dtype: str = "float32",
        tables: Optional[TableSource] = None,
    ) -> None:
        self.cuda_device_id = cuda_device_id
        self.mesh_layers = mesh_layers
        vols = _listify(volume)
        self.volumes: List[Volume] = []
        self.meshes: List[Mesh] = []
        for v in vols:
            if isinstance(v, Volume):
                self.volumes.append(v)
            elif isinstance(v, Mesh):
                self.meshes.append(v)
            else:
                raise ValueError(f"unrecognized Renderable type: {type(v)}.")
        if not self.volumes:
            raise ValueError("a projector needs at least one volume")
        if priorities is None:
            self.priorities = [len(self.volumes) - 1 - i for i in range(len(self.volumes))]
        else:
            self.priorities = []
            for prio in priorities:
                assert isinstance(prio, int), "missing priority, or priority is not an integer"
                assert 0 <= prio < len(vols), "invalid priority outside range [0, NUM_VOLUMES)"
                self.priorities.append(prio)
        assert len(self.volumes) == len(self.priorities)

        if carm is not None:
            warnings.warn("carm is deprecated, use device instead", DeprecationWarning)
            self.device = carm
        else:
            self.device = device
        self._camera_intrinsics = camera_intrinsics
        self.step = float(step)
        self.mode = mode
        self.spectrum = spectrum
        self._source_to_detector_distance = source_to_detector_distance

        if add_scatter is not None:
            log.warning("add_scatter is deprecated. Set scatter_num instead.")
            if scatter_num != 0:
                raise ValueError("Only set scatter_num.")
            self.scatter_num = 1e7 if add_scatter else 0
        elif scatter_num < 0:
            raise ValueError("scatter_num must be non-negative.")
        else:
            self.scatter_num = scatter_num
        if self.scatter_num > 0 and self.device is None:
            raise ValueError("Must provide device to simulate scatter.")
        if self.scatter_num > 0:
            raise DeprecationError("Scatter is deprecated.")

        self.add_noise = add_noise
        self.photon_count = photon_count
        self.threads = threads
        self.max_block_index = max_block_index
        self.collected_energy = collected_energy
        self.neglog = neglog
        self.intensity_upper_bound = intensity_upper_bound
        self.max_mesh_hits = max_mesh_hits
        if self.max_mesh_hits < 4 or self.max_mesh_hits % 4 != 0:
            raise ValueError("max_mesh_depth must be a multiple of 4 and >= 4")

        all_mats = []
        for v in self.volumes:
            all_mats.extend(list(v.materials[0].keys()))
        for m in self.meshes:  # projector.py:551-552
            all_mats.append(m.material)
        if attenuate_outside_volume:
            all_mats.append("air")
        self.all_materials = sorted(set(all_mats))
        # one slot per distinct mesh material, sorted (projector.py:1548-1554)
        self.mesh_materials = sorted({m.material for m in self.meshes})
        self.air_index = self.all_materials.index("air") if attenuate_outside_volume else 0
        self.attenuate_outside_volume = attenuate_outside_volume

        if density_dtype not in ("float32", "float16", "bfloat16"):
            raise ValueError(f"density_dtype must be float32, float16 or bfloat16, got {density_dtype!r}")
        self.density_dtype = density_dtype
        self._tables_source = tables
        if len(self.all_materials) > _lib.DRR_MAX_MATERIALS:
            raise ValueError(f"at most {_lib.DRR_MAX_MATERIALS} materials are supported")
        # unknown materials are rejected at construction, as the reference does (projector.py:571-577),
        # whenever a table source is known by now (given here, set as the default or named by the
        # environment); otherwise initialize() finds them when it builds the tables
        source = tables if tables is not None else configured_source()
        if source is not None:
            for mat in self.all_materials:
                if not source.has_material(mat):
                    raise ValueError(f"Material {mat} not found in material database. Please check the material name.")
        self.output_shape = None
        self.initialized = False
        self._volset = None
        self._tables = None

    # ---- properties of the reference -------------------------------------------------------
    @property
    def source_to_detector_distance(self) -> float:
        if self.device is not None:
            return self.device.source_to_detector_distance
        return self._source_to_detector_distance

    @property
    def camera_intrinsics(self) -> geo.CameraIntrinsicTransform:
        if self.device is not None:
            return self.device.camera_intrinsics
        if self._camera_intrinsics is not None:
            return self._camera_intrinsics
        raise RuntimeError("No device provided. Set the device attribute by passing `device=<device>` to the constructor.")

    @camera_intrinsics.setter
    def camera_intrinsics(self, value: geo.CameraIntrinsicTransform):
        if self.device is not None:
            raise RuntimeError("Cannot set camera intrinsics when a device is provided. Use the device's camera_intrinsics instead.")
        if not isinstance(value, geo.CameraIntrinsicTransform):
            raise TypeError(f"Expected geo.CameraIntrinsicTransform, got {type(value)} instead.")
        self._camera_intrinsics = value

    @property
    def volume(self) -> Volume:
        if len(self.volumes) != 1:
            raise AttributeError("projector contains multiple volumes. Access them with `projector.volumes[i]`")
        return self.volumes[0]

    @property
    def output_size(self) -> int:
        return int(np.prod(self.output_shape))

    # ---- lifecycle -------------------------------------------------------------------------
    def initialize(self) -> None:
        """Upload volumes (as textures) and spectrum tables to the GPU (projector.py:1395-1717)."""
        if self.initialized:
            raise RuntimeError("Close projector before initializing again.")
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("deepdrr_gb300 needs a CUDA device; there is no CPU fallback")
        lib = _lib.load()
        dev_id = 0 if self.cuda_device_id is None else int(self.cuda_device_id)
        self.torch_device = torch.device("cuda", dev_id)
        stream = torch.cuda.current_stream(self.torch_device)
        descs = (_lib.drr_volume_desc * len(self.volumes))()
        keep = []
        dtype_code = {"float32": _lib.DRR_DENSITY_F32, "float16": _lib.DRR_DENSITY_F16,
                      "bfloat16": _lib.DRR_DENSITY_BF16}[self.density_dtype]
        with torch.cuda.device(self.torch_device):
            for i, v in enumerate(self.volumes):
                ingested = v.device_arrays(self.torch_device) if hasattr(v, "device_arrays") else None
                # reference layout [i, j, k] -> texture layout [k][j][i] (projector.py:1469)
                if ingested is not None:
                    dens = ingested[0]
                else:
                    dens = torch.from_numpy(np.ascontiguousarray(v.data, dtype=np.float32)).to(self.torch_device)
                    dens = dens.permute(2, 1, 0).contiguous()
                if self.density_dtype == "float16":
                    dens = dens.half()
                elif self.density_dtype == "bfloat16":
                    dens = dens.bfloat16()
                # label remap to the sorted material list (projector.py:1495-1519)
                names, seg = v.materials
                lut = np.zeros(max(names.values()) + 1 if names else 1, dtype=np.uint8)
                for name, idx in names.items():
                    if name in self.all_materials:
                        lut[idx] = self.all_materials.index(name)
                lut_t = torch.from_numpy(lut).to(self.torch_device)
                if ingested is not None:
                    labels = lut_t[ingested[1].long()]
                else:
                    seg_t = torch.from_numpy(np.ascontiguousarray(seg.astype(np.int64))).to(self.torch_device)
                    labels = lut_t[seg_t].permute(2, 1, 0).contiguous()
                keep += [dens, labels]
                d = descs[i]
                d.density = dens.data_ptr()
                d.labels = labels.data_ptr()
                ni, nj, nk = v.shape
                d.ni, d.nj, d.nk = ni, nj, nk
                d.density_type = dtype_code
            handle = ctypes.c_void_p()
            _lib.check(lib.drr_volset_create(descs, len(self.volumes), len(self.all_materials),
                                             ctypes.c_void_p(stream.cuda_stream), ctypes.byref(handle)))
            self._volset = handle
            energies, pdf, mu = build_tables(self.spectrum, self.all_materials, self._tables_source)
            self._energies, self._pdf, self._mu = energies, pdf, mu
            th = ctypes.c_void_p()
            _lib.check(lib.drr_tables_create(energies.ctypes.data, pdf.ctypes.data, mu.ctypes.data,
                                             energies.shape[0], mu.shape[1], ctypes.c_void_p(stream.cuda_stream),
                                             ctypes.byref(th)))
            self._tables = th
        del keep
        self.output_shape = tuple(self.camera_intrinsics.sensor_size) if (
            self.device is not None or self._camera_intrinsics is not None) else None
        self.initialized = True

    def free(self) -> None:
        """Release the device copies (projector.py:1719-1764)."""
        if self.initialized:
            lib = _lib.load()
            if self._volset:
                lib.drr_volset_destroy(self._volset)
            if self._tables:
                lib.drr_tables_destroy(self._tables)
            self._volset = None
            self._tables = None
        self.initialized = False

    def __enter__(self) -> "Projector":
        self.initialize()
        return self

    def __exit__(self, type, value, tb) -> None:
        self.free()

    def __call__(self, *args, **kwargs):
        return self.project(*args, **kwargs)

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    # ---- projection ------------------------------------------------------------------------
    def _prepare_project(self, camera_projections):
        if not self.initialized:
            raise RuntimeError("Projector has not been initialized.")
        return self._views(camera_projections)

    def _views(self, camera_projections):
        """The camera projections of a call (the device's current view when none are given) and
        the maximum ray length that goes with them (projector.py:641-650)."""
        if not camera_projections and self.device is None:
            raise ValueError("must provide a camera projection object to the projector, unless imaging device "
                             "(e.g. CArm) is provided")
        if not camera_projections:
            camera_projections = [self.device.get_camera_projection()]
            self.max_ray_length = math.sqrt(self.device.source_to_detector_distance ** 2
                                            + self.device.detector_height ** 2 + self.device.detector_width ** 2)
        else:
            self.max_ray_length = self.source_to_detector_distance * 4
        return camera_projections

    def _geometry(self, camera_projections, ijk_from_world=None):
        """float64 geometry arrays of the views (world_from_index, source, IJK_from_world). An
        ``ijk_from_world`` array [n_volumes][3][4] (or [n_views][n_volumes][3][4]) replaces the
        volumes' own poses."""
        views = [geo.view_arrays(p) for p in camera_projections]
        W0, H0 = views[0][2], views[0][3]
        if any((w, h) != (W0, H0) for _, _, w, h in views):
            raise ValueError("all views of one call must share the sensor size")
        n = len(views)
        wfi = np.ascontiguousarray(np.stack([v[0] for v in views]), dtype=np.float64)
        src = np.ascontiguousarray(np.stack([v[1] for v in views]), dtype=np.float64)
        ijk = np.empty((n, len(self.volumes), 3, 4), dtype=np.float64)
        if ijk_from_world is not None:
            ijk[:] = np.asarray(ijk_from_world, dtype=np.float64)[..., :3, :4]
        else:
            for i, vol in enumerate(self.volumes):
                ijk[:, i] = np.asarray(vol.ijk_from_world.data[:3, :4])
        return W0, H0, wfi, src, ijk

    def _args(self, camera_projections, area_density, solid_angle, flags, launch, keep, ijk_from_world=None,
              outputs: bool = True):
        """drr_project_args for the views plus freshly allocated output tensors (none with
        ``outputs`` False). Every array the args point to is appended to `keep`."""
        import torch

        W0, H0, wfi, src, ijk = self._geometry(camera_projections, ijk_from_world)
        n = wfi.shape[0]
        prio = np.asarray(self.priorities, dtype=np.int32)
        enabled = np.asarray([1 if v.enabled else 0 for v in self.volumes], dtype=np.int32)
        keep += [wfi, src, ijk, prio, enabled]
        dev = self.torch_device
        M = len(self.all_materials)
        out = {}
        if outputs:
            out["intensity"] = torch.empty((n, H0, W0), dtype=torch.float32, device=dev)
            out["photon_prob"] = torch.empty((n, H0, W0), dtype=torch.float32, device=dev)
            if area_density:
                out["area_density"] = torch.empty((n, M, H0, W0), dtype=torch.float32, device=dev)
            if solid_angle or self.collected_energy:
                out["solid_angle"] = torch.empty((n, H0, W0), dtype=torch.float32, device=dev)
        a = _lib.drr_project_args()
        a.width, a.height = W0, H0
        a.step = self.step
        a.max_ray_length = float(self.max_ray_length)
        a.air_index = self.air_index
        a.flags = flags | (_lib.DRR_FLAG_ATTENUATE_OUTSIDE if self.attenuate_outside_volume else 0)
        a.n_views = n
        a.priority = prio.ctypes.data
        a.enabled = enabled.ctypes.data
        a.world_from_index = wfi.ctypes.data
        a.source_world = src.ctypes.data
        a.ijk_from_world = ijk.ctypes.data
        a.intensity = out["intensity"].data_ptr() if outputs else None
        a.photon_prob = out["photon_prob"].data_ptr() if outputs else None
        a.area_density = out["area_density"].data_ptr() if "area_density" in out else None
        a.solid_angle = out["solid_angle"].data_ptr() if "solid_angle" in out else None
        if self.meshes:
            self._mesh_args(a, wfi, src, W0, H0, keep)
        if launch:
            a.tile_warps_x = int(launch.get("tile_warps_x", 0))
            a.blocks_per_sm = int(launch.get("blocks_per_sm", 0))
            a.items_per_grab = int(launch.get("items_per_grab", 0))
        self.output_shape = (W0, H0)
        return a, out

    @property
    def _has_subtractive(self) -> bool:
        return any(m.subtractive and m.enabled for m in self.meshes)

    def _mesh_args(self, a, wfi, src, width, height, keep, stream=None) -> None:
        """Rasterise the enabled meshes for the views of `a` and point `a` at the results: additive
        integrals (drr_mesh_area_density) and, with subtractive meshes (one view per call), the
        subtractive hit lists (drr_mesh_hits) the march and the additive pass consult."""
        import torch

        n = wfi.shape[0]
        S = len(self.mesh_materials)
        out = torch.empty((n, S, height, width), dtype=torch.float32, device=self.torch_device)
        desc = self._mesh_desc(keep)
        hits = None
        if self._has_subtractive:
            if n != 1:
                raise ValueError("subtractive meshes are rendered one view per call")
            L, K = self.mesh_layers, self.max_mesh_hits
            ha = torch.empty((L, height, width, K), dtype=torch.float32, device=self.torch_device)
            hf = torch.empty((L, height, width, K), dtype=torch.int8, device=self.torch_device)
            _lib.check(_lib.load().drr_mesh_hits(ctypes.byref(desc), width, height, wfi.ctypes.data, src.ctypes.data,
                                                 K, ha.data_ptr(), hf.data_ptr(), self._stream_ptr(stream)))
            keep += [ha, hf]
            hits = (ha, hf)
            a.mesh_hit_alpha = ha.data_ptr()
            a.mesh_hit_facing = hf.data_ptr()
            a.mesh_hit_layers = L
            a.max_mesh_hits = K
        self._mesh_fill(desc, wfi, src, width, height, out, hits, stream)
        mats = np.asarray([self.all_materials.index(m) for m in self.mesh_materials], dtype=np.int32)
        keep += [out, mats]
        a.mesh_area_density = out.data_ptr()
        a.n_mesh_slots = S
        a.mesh_material = mats.ctypes.data

    def _mesh_desc(self, keep):
        """drr_mesh_desc of the enabled meshes (world-space triangles, slots, densities, layers, modes)."""
        import torch

        meshes = [m for m in self.meshes if m.enabled and len(m.faces)]
        desc = _lib.drr_mesh_desc()
        desc.n_slots = len(self.mesh_materials)
        desc.n_layers = self.mesh_layers if self._has_subtractive else 0
        if not meshes:
            desc.n_triangles = 0
            return desc
        for m in meshes:
            if m.subtractive and m.layer >= self.mesh_layers:
                raise ValueError(f"mesh layer {m.layer} >= mesh_layers ({self.mesh_layers})")
        tris = np.concatenate([m.triangles_in_world().reshape(-1, 9) for m in meshes]).astype(np.float32)
        slot = np.concatenate([np.full(len(m.faces), self.mesh_materials.index(m.material), np.int32) for m in meshes])
        dens = np.concatenate([np.full(len(m.faces), m.density, np.float32) for m in meshes])
        layer = np.concatenate([np.full(len(m.faces), m.layer, np.int32) for m in meshes])
        mode = np.concatenate([np.full(len(m.faces), (_lib.DRR_MESH_ADDITIVE if m.additive else 0)
                                       | (_lib.DRR_MESH_SUBTRACTIVE if m.subtractive else 0), np.uint8)
                               for m in meshes])
        t = [torch.from_numpy(np.ascontiguousarray(x)).to(self.torch_device) for x in (tris, slot, dens, layer, mode)]
        keep += t
        desc.triangles, desc.slot, desc.density, desc.layer, desc.mode = (x.data_ptr() for x in t)
        desc.n_triangles = len(tris)
        return desc

    def _mesh_fill(self, desc, wfi, src, width, height, out, hits=None, stream=None) -> None:
        ha, hf = hits if hits is not None else (None, None)
        _lib.check(_lib.load().drr_mesh_area_density(
            ctypes.byref(desc), width, height, wfi.shape[0], wfi.ctypes.data, src.ctypes.data,
            ha.data_ptr() if ha is not None else None, hf.data_ptr() if hf is not None else None,
            self.max_mesh_hits if ha is not None else 0, out.data_ptr(), self._stream_ptr(stream)))

    def _stream_ptr(self, stream):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream(self.torch_device)
        return ctypes.c_void_p(s.cuda_stream)

    def project_tensors(self, *camera_projections, area_density: bool = False, solid_angle: bool = False,
                        flags: int = 0, stream=None, persistent: bool = False, launch: Optional[dict] = None,
                        ijk_from_world=None) -> dict:
        """Render all views in one library call and keep the results on the GPU.

        ``persistent`` renders every view in one persistent launch (dynamic scheduling of (view,
        tile) items); ``launch`` sets its shape (keys tile_warps_x, blocks_per_sm, items_per_grab,
        e.g. from :meth:`autotune`). Returns torch tensors: ``intensity`` and ``photon_prob``
        [N, H, W] (float32), and optionally ``area_density`` [N, M, H, W] (g/cm^2) and
        ``solid_angle`` [N, H, W]. ``ijk_from_world`` ([n_volumes][3][4], float64) replaces the
        volumes' poses for this call."""
        camera_projections = self._prepare_project(camera_projections)
        if self._has_subtractive and len(camera_projections) > 1:
            # subtractive hit lists are built per view (projector.py:709-716 renders meshes per view)
            import torch

            parts = [self.project_tensors(p, area_density=area_density, solid_angle=solid_angle, flags=flags,
                                          stream=stream, ijk_from_world=ijk_from_world) for p in camera_projections]
            return {k: torch.cat([q[k] for q in parts]) for k in parts[0]}
        keep = []
        a, out = self._args(camera_projections, area_density, solid_angle,
                            flags | (_lib.DRR_FLAG_PERSISTENT if persistent else 0), launch, keep, ijk_from_world)
        _lib.check(_lib.load().drr_project(self._volset, self._tables, ctypes.byref(a), self._stream_ptr(stream)))
        return out

    def set_density(self, density, volume: int = 0, stream=None) -> None:
        """Replace the densities of one volume from a CUDA tensor [ni, nj, nk] (the reference's
        layout), keeping its labels; float32 and float16 volumes."""
        import torch

        if not self.initialized:
            raise RuntimeError("Projector has not been initialized.")
        ni, nj, nk = self.volumes[volume].shape
        if tuple(density.shape) != (ni, nj, nk):
            raise ValueError(f"density shape {tuple(density.shape)} != volume shape {(ni, nj, nk)}")
        dt = {"float32": torch.float32, "float16": torch.float16}.get(self.density_dtype)
        if dt is None:
            raise ValueError("set_density supports float32 and float16 volumes")
        dens = density.detach().to(device=self.torch_device, dtype=dt).permute(2, 1, 0).contiguous()
        s = stream if stream is not None else torch.cuda.current_stream(self.torch_device)
        _lib.check(_lib.load().drr_volset_set_density(self._volset, int(volume), dens.data_ptr(),
                                                      ctypes.c_void_p(s.cuda_stream)))
        dens.record_stream(s)

    def project_adjoint(self, *camera_projections, area_density=None, grad_intensity=None, grad_photon_prob=None,
                        grad_area_density=None, density: bool = True, pose: bool = False, center=None,
                        ijk_from_world=None, stream=None) -> dict:
        """Gradients of a loss through :meth:`project_tensors` (one volume, no air attenuation).

        Upstream gradients are CUDA tensors shaped like the forward's outputs; ``area_density`` is
        the forward's [N, M, H, W] output for the same views (None: recomputed). Returns
        ``density``: dL/d(density) [ni, nj, nk] float32, and with ``pose`` ``pose``: [N, 6]
        dL/d(translation, rotation vector) of a rigid motion of the volume about ``center``
        (world, default the volume's centre), per view."""
        import torch

        camera_projections = self._prepare_project(camera_projections)
        keep = []
        a, _ = self._args(camera_projections, False, False, 0, None, keep, ijk_from_world, outputs=False)
        n = a.n_views
        ni, nj, nk = self.volumes[0].shape
        dev = self.torch_device
        out = {}
        adj = _lib.drr_adjoint_args()

        def ptr(t, name):
            if t is None:
                return None
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
                raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
            keep.append(t)
            return t.data_ptr()

        adj.area_density = ptr(area_density, "area_density")
        adj.grad_intensity = ptr(grad_intensity, "grad_intensity")
        adj.grad_photon_prob = ptr(grad_photon_prob, "grad_photon_prob")
        adj.grad_area_density = ptr(grad_area_density, "grad_area_density")
        if density:
            out["density"] = torch.zeros((nk, nj, ni), dtype=torch.float32, device=dev)
            adj.grad_density = out["density"].data_ptr()
        if pose:
            out["pose"] = torch.zeros((n, 6), dtype=torch.float32, device=dev)
            adj.grad_pose = out["pose"].data_ptr()
        c = self.volume_center_world(0) if center is None else np.asarray(center, dtype=np.float64)
        for k in range(3):
            adj.center[k] = float(c[k])
        _lib.check(_lib.load().drr_project_adjoint(self._volset, self._tables, ctypes.byref(a), ctypes.byref(adj),
                                                   self._stream_ptr(stream)))
        if density:
            out["density"] = out["density"].permute(2, 1, 0)
        return out

    def volume_center_world(self, volume: int = 0) -> np.ndarray:
        """World position of the centre of a volume's voxel grid."""
        v = self.volumes[volume]
        ijk = (np.asarray(v.shape, dtype=np.float64) - 1.0) / 2.0
        wfi = np.linalg.inv(np.asarray(v.ijk_from_world.data, dtype=np.float64))
        return (wfi @ np.append(ijk, 1.0))[:3]

    def autotune(self, *camera_projections, max_views: int = 32, stream=None, cache: bool = True) -> dict:
        """Fastest persistent launch shape for these views (cached per GPU, volumes, materials,
        detector size and view count in ~/.cache/deepdrr_gb300/autotune.json)."""
        import json
        import os
        import torch

        camera_projections = self._prepare_project(camera_projections)
        W0, H0 = geo.view_arrays(camera_projections[0])[2:]
        key = "|".join(str(x) for x in (torch.cuda.get_device_name(self.torch_device),
                                          [v.shape for v in self.volumes], len(self.all_materials), W0, H0,
                                          min(len(camera_projections), max_views), self.density_dtype))
        path = Path(os.environ.get("DEEPDRR_GB300_CACHE", Path.home() / ".cache" / "deepdrr_gb300")) / "autotune.json"
        table = {}
        if cache and path.exists():
            try:
                table = json.loads(path.read_text())
            except (OSError, ValueError):
                table = {}
        if key in table:
            return table[key]
        keep = []
        a, _ = self._args(camera_projections, False, False, _lib.DRR_FLAG_PERSISTENT, None, keep)
        r = _lib.drr_tune_result()
        _lib.check(_lib.load().drr_autotune(self._volset, self._tables, ctypes.byref(a), int(max_views),
                                            self._stream_ptr(stream), ctypes.byref(r)))
        best = dict(tile_warps_x=r.tile_warps_x, blocks_per_sm=r.blocks_per_sm, items_per_grab=r.items_per_grab,
                    ms_per_view=r.ms_per_view)
        if cache:
            table[key] = best
            try:
                path.parent.mkdir(parents=True, exist_ok=True)
                path.write_text(json.dumps(table, indent=1))
            except OSError:
                pass
        return best

    def capture(self, *camera_projections, area_density: bool = False, launch: Optional[dict] = None) -> "ProjectionGraph":
        """Capture a persistent projection of these views in a CUDA graph (see ProjectionGraph)."""
        camera_projections = self._prepare_project(camera_projections)
        return ProjectionGraph(self, camera_projections, area_density, launch)

    def project(self, *camera_projections) -> np.ndarray:
        """Render, post-process and return numpy float32 [H, W] (one view) or [N, H, W]."""
        images = self.project_images(*camera_projections)
        images = images.cpu().numpy()
        return images[0] if images.shape[0] == 1 else images

    def project_images(self, *camera_projections, stream=None):
        """``project`` without the host copy: the post-processed [N, H, W] float32 images on the GPU."""
        import torch

        out = self.project_tensors(*camera_projections, stream=stream)
        images = out["intensity"]
        if self.collected_energy:
            images = self._collected_energy(camera_projections, images, out["solid_angle"], stream)
        lib = _lib.load()
        s = stream if stream is not None else torch.cuda.current_stream(self.torch_device)
        sp = ctypes.c_void_p(s.cuda_stream)
        n, h, w = images.shape
        if self.add_noise:
            # projector.py:691-695: shot noise from photon_prob * photon_count. The seed is drawn
            # from numpy's global generator, which the reference's np.random.poisson also uses, so
            # np.random.seed makes a run repeatable in the same way.
            seed = int(np.random.randint(0, 2 ** 63 - 1, dtype=np.int64))
            noisy = torch.empty_like(images)
            _lib.check(lib.drr_add_noise(images.data_ptr(), out["photon_prob"].data_ptr(), noisy.data_ptr(), n, h, w,
                                         float(self.photon_count), seed, sp))
            images = noisy
        if self.intensity_upper_bound is not None:
            _lib.check(lib.drr_clip_upper(images.data_ptr(), images.numel(), float(self.intensity_upper_bound), sp))
        if self.neglog:
            _lib.check(lib.drr_neglog(images.data_ptr(), n, h * w, 0.01, sp))
        return images

    def _collected_energy(self, camera_projections, intensity, solid_angle, stream=None):
        """projector.py:833-853 on the GPU (drr_collected_energy): intensity * solid angle * photons /
        mean(solid angle) / pixel area, keV per mm^2."""
        import torch

        projs = self._prepare_project(camera_projections)
        area = np.ascontiguousarray([(self.source_to_detector_distance / proj.intrinsic.fx)
                                     * (self.source_to_detector_distance / proj.intrinsic.fy) for proj in projs],
                                    dtype=np.float64)
        n, h, w = intensity.shape
        out = torch.empty_like(intensity)
        _lib.check(_lib.load().drr_collected_energy(intensity.data_ptr(), solid_angle.contiguous().data_ptr(),
                                                    out.data_ptr(), n, h * w, float(self.photon_count),
                                                    area.ctypes.data, self._stream_ptr(stream)))
        return out


class ProjectionGraph:
    """A persistent projection of a fixed number of views captured in a CUDA graph.

    The graph holds the upload of the view records, the reset of the work counter and the
    persistent kernel; ``launch()`` replays it into the same output tensors, ``set_views(...)``
    replaces the view geometry (same number of views and sensor size) before the next replay.
    """

    def __init__(self, projector: Projector, camera_projections, area_density: bool, launch: Optional[dict]):
        if projector._has_subtractive:
            raise NotImplementedError("subtractive meshes are rendered one view per call, not in a graph")
        self.projector = projector
        self._keep = []
        self.args, self.outputs = projector._args(camera_projections, area_density, False,
                                                  _lib.DRR_FLAG_PERSISTENT, launch, self._keep)
        if projector.meshes:
            import torch

            n, S = self.args.n_views, len(projector.mesh_materials)
            buf = [t for t in self._keep if isinstance(t, torch.Tensor) and t.data_ptr() == self.args.mesh_area_density]
            self.outputs = dict(self.outputs, _mesh_area_density=buf[0])
        self.n_views = self.args.n_views
        handle = ctypes.c_void_p()
        _lib.check(_lib.load().drr_graph_create(projector._volset, projector._tables, ctypes.byref(self.args),
                                                ctypes.byref(handle)))
        self._graph = handle

    def set_views(self, *camera_projections) -> None:
        W0, H0, wfi, src, ijk = self.projector._geometry(camera_projections)
        if wfi.shape[0] != self.n_views or (W0, H0) != (self.args.width, self.args.height):
            raise ValueError("a captured projection keeps its number of views and sensor size")
        if self.projector.meshes:
            # the graph reads the mesh integrals from a fixed buffer: rasterise the new views into it
            out = self.outputs["_mesh_area_density"]
            self.projector._mesh_fill(self.projector._mesh_desc(self._keep), wfi, src, W0, H0, out)
        _lib.check(_lib.load().drr_graph_set_views(self._graph, wfi.ctypes.data, src.ctypes.data, ijk.ctypes.data))

    def launch(self, stream=None) -> dict:
        _lib.check(_lib.load().drr_graph_launch(self._graph, self.projector._stream_ptr(stream)))
        return {k: v for k, v in self.outputs.items() if not k.startswith("_")}

    def close(self) -> None:
        if self._graph:
            _lib.load().drr_graph_destroy(self._graph)
            self._graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
