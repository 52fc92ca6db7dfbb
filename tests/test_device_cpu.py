"""CPU tests of the X-ray devices (deepdrr_gb300.device): the properties the reference's
SimpleDevice / MobileCArm definitions imply (deepdrr/device/simple_device.py,
mobile_carm.py), checked on the camera projections they produce."""
import math
from pathlib import Path

import numpy as np
import pytest

from deepdrr_gb300 import Projector
from deepdrr_gb300.device import CameraProjectionDevice, MobileCArm, SimpleDevice, pose_vector_angles
from deepdrr_gb300.geo import FrameTransform, view_arrays


def project_point(proj, x):
    h = proj.index_from_world @ np.append(np.asarray(x, dtype=np.float64), 1.0)
    return h[:2] / h[2]


def test_simple_device_default_view():
    d = SimpleDevice(sensor_height=300, sensor_width=400, pixel_size=0.5, source_to_detector_distance=1000.0)
    proj = d.get_camera_projection()
    # the default view looks along +z at the origin, the origin halfway between source and detector
    np.testing.assert_allclose(proj.center_in_world, [0.0, 0.0, -500.0], atol=1e-9)
    np.testing.assert_allclose(project_point(proj, [0.0, 0.0, 0.0]), [200.0, 150.0], atol=1e-9)
    np.testing.assert_allclose(d.principle_ray_in_world, [0.0, 0.0, 1.0], atol=1e-12)
    assert d.detector_width == 200.0 and d.detector_height == 150.0
    K = d.camera_intrinsics.data
    assert K[0, 0] == 2000.0 and K[0, 2] == 200.0 and K[1, 2] == 150.0


@pytest.mark.parametrize("direction,up", [([1.0, 0.2, -0.3], [0.0, 0.0, 1.0]), ([0.0, 1.0, 0.0], [0.0, 0.0, 1.0]),
                                          ([-0.3, -0.4, 0.8], [1.0, 0.0, 0.0])])
def test_simple_device_set_view(direction, up):
    d = SimpleDevice(sensor_height=256, sensor_width=256, pixel_size=1.0, source_to_detector_distance=1000.0)
    point = np.array([10.0, -20.0, 30.0])
    d.set_view(point, direction, up, source_to_point_fraction=0.7)
    proj = d.get_camera_projection()
    dn = np.asarray(direction) / np.linalg.norm(direction)
    np.testing.assert_allclose(proj.center_in_world, point - 700.0 * dn, atol=1e-8)
    np.testing.assert_allclose(project_point(proj, point), [128.0, 128.0], atol=1e-8)
    # the up vector points towards -v in the image
    uv = project_point(proj, point + 10.0 * np.asarray(up))
    assert uv[1] < 128.0 - 1.0
    assert abs(uv[0] - 128.0) < 1e-6 + 1e-9 * abs(uv[1])


def test_simple_device_keeps_the_ray_frame_when_up_is_antiparallel_to_it():
    """simple_device.py:142-147: the in-plane turn is skipped when the projected up vector is
    parallel or antiparallel to the ray frame's -y; with direction +y that frame's -y is +z, so an
    up of -z is left pointing along +v (the reference's behaviour, kept)."""
    d = SimpleDevice(sensor_height=64, sensor_width=64, pixel_size=1.0, source_to_detector_distance=1000.0)
    d.set_view([0.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, -1.0])
    uv = project_point(d.get_camera_projection(), [0.0, 0.0, -10.0])
    assert uv[1] > 32.0 + 1.0


def test_simple_device_scale_sensor():
    d = SimpleDevice(sensor_height=200, sensor_width=400)
    d.scale_sensor(300.0)
    assert d.pixel_size == 1.5


def test_mobile_carm_neutral_pose():
    c = MobileCArm()
    assert c.source_to_detector_distance == 1020.0
    np.testing.assert_allclose(c.source_in_device, [0.0, 0.0, -530.0])
    np.testing.assert_allclose(c.principle_ray, [0.0, 0.0, 1.0])
    proj = c.get_camera_projection()
    np.testing.assert_allclose(proj.center_in_world, [0.0, 0.0, -530.0], atol=1e-9)
    np.testing.assert_allclose(project_point(proj, [0.0, 0.0, 0.0]), [768.0, 768.0], atol=1e-9)
    # rotate_camera_left turns the camera 90 degrees about the principal ray: device +x runs along +v
    uv = project_point(proj, [10.0, 0.0, 0.0])
    assert abs(uv[0] - 768.0) < 1e-6 and uv[1] > 768.0
    uv = project_point(MobileCArm(rotate_camera_left=False).get_camera_projection(), [10.0, 0.0, 0.0])
    assert abs(uv[1] - 768.0) < 1e-6 and uv[0] > 768.0


def test_mobile_carm_rotations_and_isocenter():
    c = MobileCArm(isocenter=[5.0, -3.0, 2.0], alpha=30.0, beta=-20.0)
    a, b = math.radians(30.0), math.radians(-20.0)
    Rx = np.array([[1, 0, 0], [0, math.cos(a), -math.sin(a)], [0, math.sin(a), math.cos(a)]])
    Ry = np.array([[math.cos(b), 0, math.sin(b)], [0, 1, 0], [-math.sin(b), 0, math.cos(b)]])
    R = Ry @ Rx  # alpha about x first, then beta about the fixed y axis
    np.testing.assert_allclose(c.source_in_device, R @ [0.0, 0.0, -530.0] + [5.0, -3.0, 2.0], atol=1e-9)
    np.testing.assert_allclose(c.principle_ray, R @ [0.0, 0.0, 1.0], atol=1e-12)
    proj = c.get_camera_projection()
    np.testing.assert_allclose(project_point(proj, c.isocenter), [768.0, 768.0], atol=1e-8)
    # pose_vector_angles inverts the angles of the principal ray
    al, be = pose_vector_angles(c.principle_ray)
    assert abs(al - a) < 1e-12 and abs(be - b) < 1e-12


def test_mobile_carm_moves_and_bounds():
    c = MobileCArm()
    c.move_by(delta_alpha=200.0)
    assert abs(c.alpha - math.radians(110.0)) < 1e-12  # clipped at max_alpha
    c.move_to(alpha=10.0, beta=5.0, gamma=3.0)
    assert abs(c.beta - math.radians(5.0)) < 1e-12 and abs(c.gamma - math.radians(3.0)) < 1e-12
    ray = np.array([0.3, -0.2, 0.9])
    c.move_to(principle_ray_in_world=ray)
    np.testing.assert_allclose(c.principle_ray, ray / np.linalg.norm(ray), atol=1e-12)
    c.move_to(isocenter_in_world=[1.0, 2.0, 3.0])
    np.testing.assert_allclose(c.isocenter, [1.0, 2.0, 3.0])
    with pytest.raises(ValueError):
        MobileCArm(isocenter=[500.0, 0.0, 0.0], enforce_isocenter_bounds=True)
    c2 = MobileCArm(**c.to_config())
    np.testing.assert_allclose(c2.get_camera_projection().index_from_world, c.get_camera_projection().index_from_world)


def test_mobile_carm_reposition_and_world_frame():
    c = MobileCArm(source_to_isocenter_horizontal_offset=20.0)
    c.reposition(viewpoint_in_world=[100.0, 50.0, -10.0])
    np.testing.assert_allclose(c.viewpoint_in_world, [100.0, 50.0, -10.0], atol=1e-9)
    proj = c.get_camera_projection()
    np.testing.assert_allclose(project_point(proj, c.viewpoint_in_world), [768.0, 768.0], atol=1e-8)
    # the whole device placed by world_from_device: projections follow the transform
    T = FrameTransform.from_rt(np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1.0]]), [5.0, 6.0, 7.0])
    c3 = MobileCArm(world_from_device=T, alpha=15.0)
    c4 = MobileCArm(alpha=15.0)
    x = np.array([3.0, -4.0, 12.0])
    np.testing.assert_allclose(project_point(c3.get_camera_projection(), T @ x),
                               project_point(c4.get_camera_projection(), x), atol=1e-8)


def test_camera_projection_device_round_trip():
    c = MobileCArm(alpha=20.0, beta=10.0)
    proj = c.get_camera_projection()
    d = CameraProjectionDevice(proj, pixel_size=0.194)
    assert abs(d.source_to_detector_distance - 1020.0) < 1e-9
    np.testing.assert_allclose(d.get_camera_projection().index_from_world, proj.index_from_world, atol=1e-9)


def test_projector_takes_its_view_from_a_device():
    from deepdrr_gb300.phantoms import simple_phantom_hu, volume_from_hu

    vol = volume_from_hu(simple_phantom_hu(16, seed=1))
    c = MobileCArm(sensor_height=32, sensor_width=48, pixel_size=4.0)
    p = Projector(vol, device=c)
    projs = p._views(())
    W, s, w, h = view_arrays(projs[0])
    W2, s2, _, _ = view_arrays(c.get_camera_projection())
    np.testing.assert_allclose(W, W2)
    np.testing.assert_allclose(s, s2)
    assert (w, h) == (48, 32)
    assert abs(p.max_ray_length - math.sqrt(1020.0 ** 2 + (32 * 4.0) ** 2 + (48 * 4.0) ** 2)) < 1e-9


# ---- pinned to the reference's own device classes -------------------------------------------------

DEVICE_GOLDEN = Path(__file__).resolve().parent / "golden" / "device_reference.npz"


def _replay(sc):
    from deepdrr_gb300.device import MobileCArm, SimpleDevice
    from deepdrr_gb300.geo import FrameTransform

    init = dict(sc["init"])
    if "world_from_device" in init:
        init["world_from_device"] = FrameTransform(np.array(init["world_from_device"]))
    d = SimpleDevice(**init) if sc["kind"] == "simple" else MobileCArm(**init)
    for name, kw in sc["ops"]:
        getattr(d, name)(**kw)
    return d


def test_devices_reproduce_the_reference_device_classes():
    """camera3d_from_world, intrinsics and C-arm state of this package's SimpleDevice / MobileCArm
    against the reference's own classes (deepdrr/device/simple_device.py, mobile_carm.py) run on the
    same seeded scenarios by tests/golden/make_device_vectors.py (killeengeo replaced by
    tests/golden/geo_standin.py): equal to 1e-9."""
    import json

    g = np.load(DEVICE_GOLDEN)
    scs = json.loads(str(g["scenarios"]))
    assert len(scs) >= 20
    for i, sc in enumerate(scs):
        d = _replay(sc)
        np.testing.assert_allclose(np.asarray(d.camera3d_from_world.data), g[f"s{i}__camera3d_from_world"],
                                   rtol=0, atol=1e-9, err_msg=f"scenario {i} ({sc['kind']})")
        np.testing.assert_allclose(np.asarray(d.camera_intrinsics.data), g[f"s{i}__intrinsic"], rtol=1e-15, atol=0)
        if sc["kind"] == "carm":
            np.testing.assert_allclose(d.isocenter, g[f"s{i}__isocenter"], rtol=0, atol=1e-9)
            np.testing.assert_allclose([d.alpha, d.beta, d.gamma], g[f"s{i}__angles"], rtol=0, atol=1e-12)
