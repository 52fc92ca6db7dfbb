"""CPU tests of the Projector's host-side behaviour (argument checks and errors mirror
deepdrr/projector/projector.py:398-587, 628-652)."""
import numpy as np
import pytest

import deepdrr_gb300 as dd
from deepdrr_gb300 import geo
from deepdrr_gb300.phantoms import volume_from_hu, simple_phantom_hu

from helpers import uniform_cube


def _vol():
    return volume_from_hu(simple_phantom_hu(16, seed=1))


def test_default_priorities_make_the_last_volume_win():
    p = dd.Projector([_vol(), _vol(), _vol()])
    assert p.priorities == [2, 1, 0]


def test_priorities_are_checked():
    with pytest.raises(AssertionError):
        dd.Projector([_vol(), _vol()], priorities=[0, 2])
    with pytest.raises(AssertionError):
        dd.Projector([_vol(), _vol()], priorities=[0, 1.0])


def test_material_list_is_sorted_and_air_added_for_attenuation():
    v = uniform_cube(8, material="bone")
    p = dd.Projector([v, _vol()])
    assert p.all_materials == ["air", "bone", "soft tissue"]
    p = dd.Projector(v, attenuate_outside_volume=True)
    assert p.all_materials == ["air", "bone"] and p.air_index == 0


def test_deprecated_and_invalid_options_raise():
    with pytest.raises(dd.DeprecationError):
        dd.Projector(_vol(), scatter_num=10, device=object())
    with pytest.raises(ValueError):
        dd.Projector(_vol(), scatter_num=10)
    with pytest.raises(ValueError):
        dd.Projector(_vol(), scatter_num=-1)
    with pytest.raises(ValueError):
        dd.Projector(_vol(), max_mesh_hits=6)
    with pytest.raises(ValueError):
        dd.Projector(_vol(), add_scatter=True, scatter_num=3)
    with pytest.raises(ValueError):
        dd.Projector("not a volume")


def test_unknown_material_raises_at_construction():
    """projector.py:571-577: a material missing from the attenuation tables is a ValueError when the
    projector is built (here against the default table source the test session configures)."""
    n = 8
    v = dd.Volume.from_parameters(np.ones((n, n, n), np.float32), {"unobtainium": np.ones((n, n, n), bool)},
                                  origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0))
    with pytest.raises(ValueError, match="unobtainium"):
        dd.Projector(v)
    dd.Projector(uniform_cube(n, material="bone"))  # a known material passes


def test_project_before_initialize_raises():
    p = dd.Projector(_vol())
    with pytest.raises(RuntimeError):
        p.project()


def test_single_volume_property():
    assert isinstance(dd.Projector(_vol()).volume, dd.Volume)
    with pytest.raises(AttributeError):
        dd.Projector([_vol(), _vol()]).volume


def test_camera_projection_round_trip():
    proj = geo.CameraProjection.from_view((10.0, -5.0, 3.0), (0.2, 1.0, -0.1), (0, 0, 1),
                                          source_to_detector_distance=1020.0, pixel_size=0.5, sensor_size=(64, 48))
    W = np.asarray(proj.world_from_index)[:3]
    P = proj.index_from_world
    s = proj.center_in_world
    for u, v in [(0.5, 0.5), (31.5, 20.5), (63.5, 47.5)]:
        x = s + W @ np.array([u, v, 1.0])
        h = P @ np.append(x, 1.0)
        assert h[0] / h[2] == pytest.approx(u) and h[1] / h[2] == pytest.approx(v)
    assert proj.sensor_width == 64 and proj.sensor_height == 48
    # principal ray points along the view direction
    d = W @ np.array([32.0, 24.0, 1.0])
    d /= np.linalg.norm(d)
    ref = np.array([0.2, 1.0, -0.1]) / np.linalg.norm([0.2, 1.0, -0.1])
    assert np.allclose(d, ref)


def test_hu_conversion_and_thresholds():
    hu = np.array([-1000.0, -800.0, -799.0, 0.0, 350.0, 351.0, 2000.0])
    d = dd.hu_to_density(hu)
    assert np.allclose(d, np.maximum(np.minimum(0.001029 * hu + 1.030, 0.0005886 * hu + 1.03), 0))
    m = dd.segment_thresholds(hu)
    assert m["air"].tolist() == [True, True, False, False, False, False, False]
    assert m["bone"].tolist() == [False] * 5 + [True, True]
    names, seg = dd.format_materials({"a": np.array([1, 1, 0]), "b": np.array([0, 1, 1])})
    assert names == {"a": 0, "b": 1} and seg.tolist() == [0, 1, 1]
