"""Golden poses of the reference's own device classes, for tests/test_device_cpu.py.

Runs deepdrr/device/{device,simple_device,mobile_carm}.py from the reference sources as they stand,
with tests/golden/geo_standin.py in place of killeengeo (not installed here) and small stubs for
the modules they import only for meshes and bookkeeping (pyvista; deepdrr.utils.radians, which
converts degrees to radians), over seeded scenarios: SimpleDevice.set_view with points, directions
and up vectors (parallel and antiparallel cases included) under a rotated world_from_device, and
MobileCArm poses, rotations with and without rotate_camera_left, move_by / move_to (with
isocenter_in_world, interest_point_in_world and principle_ray_in_world) and reposition. For every
scenario it records camera3d_from_world (4x4), the intrinsic matrix and, for the C-arm, the
isocenter and angles. Those pin the reference's frame composition; killeengeo's own arithmetic
stays unpinned (see geo_standin.py).

    python tests/golden/make_device_vectors.py [--reference PATH] [--out tests/golden/device_reference.npz]
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import math
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (ROOT, HERE):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

from oracle.build_ref import default_reference  # noqa: E402


def rigid(rng, t_mm, deg):
    from scipy.spatial.transform import Rotation

    T = np.eye(4)
    T[:3, :3] = Rotation.from_rotvec(rng.normal(size=3) / np.sqrt(3) * np.deg2rad(deg)).as_matrix()
    T[:3, 3] = rng.uniform(-1, 1, 3) * t_mm
    return T


def scenarios():
    """Seeded scenarios as plain data, replayed on both implementations."""
    rng = np.random.default_rng(7)
    out = []
    out.append(dict(kind="simple", init=dict(), ops=[]))
    for k in range(6):
        init = dict(sensor_height=int(rng.integers(64, 512)), sensor_width=int(rng.integers(64, 512)),
                    pixel_size=float(rng.uniform(0.2, 1.5)), source_to_detector_distance=float(rng.uniform(800, 1200)),
                    world_from_device=rigid(rng, 200, 40).tolist())
        d = rng.normal(size=3)
        ops = [("set_view", dict(point=rng.uniform(-50, 50, 3).tolist(), direction=d.tolist(),
                                 up=rng.normal(size=3).tolist(), source_to_point_distance=float(rng.uniform(300, 700))))]
        if k % 2:
            ops.append(("set_view", dict(point=None, direction=rng.normal(size=3).tolist(), up=None,
                                         source_to_point_fraction=float(rng.uniform(0.3, 0.8)))))
        out.append(dict(kind="simple", init=init, ops=ops))
    # direction along +z and -z in the device frame; up along and against the ray frame's -y
    out.append(dict(kind="simple", init=dict(), ops=[("set_view", dict(point=[1, 2, 3], direction=[0, 0, 1],
                                                                       up=[0, -1, 0]))]))
    out.append(dict(kind="simple", init=dict(), ops=[("set_view", dict(point=[1, 2, 3], direction=[0, 0, -2],
                                                                       up=[0, 1, 0]))]))
    out.append(dict(kind="simple", init=dict(), ops=[("set_view", dict(point=[0, 0, 0], direction=[1, 0, 0],
                                                                       up=[0, 1, 0]))]))
    out.append(dict(kind="carm", init=dict(), ops=[]))
    for k in range(8):
        init = dict(alpha=float(rng.uniform(-30, 100)), beta=float(rng.uniform(-60, 60)),
                    gamma=float(rng.uniform(-20, 20)), isocenter=rng.uniform(-80, 80, 3).tolist(),
                    rotate_camera_left=bool(k % 2), source_to_isocenter_horizontal_offset=float(rng.uniform(-20, 20)),
                    world_from_device=rigid(rng, 300, 30).tolist())
        ops = []
        if k % 3 == 0:
            ops.append(("move_by", dict(delta_isocenter=rng.uniform(-10, 10, 3).tolist(),
                                        delta_alpha=float(rng.uniform(-10, 10)), delta_beta=float(rng.uniform(-10, 10)),
                                        delta_gamma=float(rng.uniform(-5, 5)))))
        if k % 3 == 1:
            ops.append(("move_to", dict(alpha=float(rng.uniform(-30, 90)), beta=float(rng.uniform(-40, 40)),
                                        interest_point_in_world=rng.uniform(-50, 50, 3).tolist())))
            ops.append(("move_to", dict(isocenter_in_world=rng.uniform(-60, 60, 3).tolist(), gamma=10.0)))
        if k % 3 == 2:
            ops.append(("move_to", dict(principle_ray_in_world=rng.normal(size=3).tolist(), gamma=7.0)))
            ops.append(("reposition", dict(viewpoint_in_world=rng.uniform(-100, 100, 3).tolist())))
        out.append(dict(kind="carm", init=init, ops=ops))
    # alpha and beta beyond their limits are clipped
    out.append(dict(kind="carm", init=dict(alpha=150.0, beta=-300.0), ops=[]))
    return out


def load_reference(reference: Path):
    import geo_standin

    root = reference / "deepdrr"
    pkg = types.ModuleType("deepdrr")
    pkg.__path__ = [str(root)]
    sys.modules["deepdrr"] = pkg
    sys.modules["deepdrr.geo"] = geo_standin
    pkg.geo = geo_standin
    sys.modules["killeengeo"] = geo_standin
    sys.modules["pyvista"] = types.ModuleType("pyvista")
    utils = types.ModuleType("deepdrr.utils")

    def radians(*args, degrees=True):
        if len(args) != 1:
            raise NotImplementedError("one angle at a time")
        t = args[0]
        return math.radians(t) if degrees else t

    utils.radians = radians
    utils.jsonable = lambda x: x
    utils.try_import_pyvista = lambda: (None, False)
    sys.modules["deepdrr.utils"] = utils
    pkg.utils = utils
    dev = types.ModuleType("deepdrr.device")
    dev.__path__ = [str(root / "device")]
    sys.modules["deepdrr.device"] = dev
    mods = {}
    for name in ("device", "simple_device", "mobile_carm"):
        spec = importlib.util.spec_from_file_location(f"deepdrr.device.{name}", root / "device" / f"{name}.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"deepdrr.device.{name}"] = mod
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods["simple_device"].SimpleDevice, mods["mobile_carm"].MobileCArm, geo_standin


def run_reference(SimpleDevice, MobileCArm, geo, sc):
    init = dict(sc["init"])
    if "world_from_device" in init:
        init["world_from_device"] = geo.frame_transform(np.array(init["world_from_device"]))
    d = SimpleDevice(**init) if sc["kind"] == "simple" else MobileCArm(**init)
    for name, kw in sc["ops"]:
        kw = dict(kw)
        for key in ("interest_point_in_world", "viewpoint_in_world"):  # the reference takes Point3D here
            if kw.get(key) is not None:
                kw[key] = geo.point(kw[key])
        getattr(d, name)(**kw)
    out = dict(camera3d_from_world=np.array(d.camera3d_from_world.data),
               intrinsic=np.array(d.camera_intrinsics.data))
    if sc["kind"] == "carm":
        out.update(isocenter=np.array(d.isocenter), angles=np.array([d.alpha, d.beta, d.gamma], dtype=np.float64))
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(default_reference()))
    ap.add_argument("--out", default=str(HERE / "device_reference.npz"))
    args = ap.parse_args()
    SimpleDevice, MobileCArm, geo = load_reference(Path(args.reference))
    rec = {"scenarios": np.array(json.dumps(scenarios()))}
    for i, sc in enumerate(scenarios()):
        for k, v in run_reference(SimpleDevice, MobileCArm, geo, sc).items():
            rec[f"s{i}__{k}"] = v
    np.savez_compressed(args.out, **rec)
    print(f"wrote {args.out}: {len(scenarios())} scenarios")


if __name__ == "__main__":
    main()
