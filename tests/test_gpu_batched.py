"""GPU tests of the batched paths: the persistent (view, tile) kernel, its CUDA-graph capture and
its launch-shape autotuner, all against the plain per-launch kernel (bit-identical results)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import deepdrr_gb300 as dd
from deepdrr_gb300 import tables
from deepdrr_gb300.phantoms import implant_volume, random_rigid, random_views, simple_phantom_hu, volume_from_hu

from helpers import GOLDEN_TABLES

pytestmark = pytest.mark.gpu


def _scene(nvol, views=5, sensor=(40, 36)):
    rng = np.random.default_rng(21)
    a = volume_from_hu(simple_phantom_hu(40, seed=21))
    vols = [a]
    if nvol >= 2:
        b = volume_from_hu(simple_phantom_hu(24, seed=22), spacing=(1.3, 1.3, 1.3))
        b.world_from_anatomical = random_rigid(rng, 8.0, 20.0)
        vols.append(b)
    if nvol >= 3:
        c = implant_volume((16, 16, 12), seed=23)
        c.world_from_anatomical = random_rigid(rng, 5.0, 30.0)
        vols.append(c)
    projs = random_views(views, a.center_in_world, seed=24, sphere_mm=5.0, sensor_size=sensor, pixel_size=2.0)
    return vols, projs


def _projector(vols):
    p = dd.Projector(vols, spectrum="90KV_AL40", tables=tables.NpzTables(GOLDEN_TABLES), neglog=False)
    p.initialize()
    return p


def _np(out):
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("nvol", [1, 3])
@pytest.mark.parametrize("launch", [None, dict(tile_warps_x=1, blocks_per_sm=3, items_per_grab=1),
                                    dict(tile_warps_x=4, blocks_per_sm=1, items_per_grab=4)])
def test_persistent_equals_plain(nvol, launch):
    vols, projs = _scene(nvol)
    p = _projector(vols)
    try:
        plain = _np(p.project_tensors(*projs, area_density=True))
        pers = _np(p.project_tensors(*projs, area_density=True, persistent=True, launch=launch))
    finally:
        p.free()
    for k in plain:
        np.testing.assert_array_equal(plain[k], pers[k])


def test_many_views_in_one_persistent_launch():
    vols, projs = _scene(2, views=70, sensor=(24, 20))  # more views than one plain launch holds
    p = _projector(vols)
    try:
        plain = _np(p.project_tensors(*projs))
        pers = _np(p.project_tensors(*projs, persistent=True))
    finally:
        p.free()
    np.testing.assert_array_equal(plain["intensity"], pers["intensity"])


def test_graph_replay_and_new_views():
    vols, projs = _scene(3, views=6)
    other = random_views(6, vols[0].center_in_world, seed=99, sphere_mm=5.0, sensor_size=(40, 36), pixel_size=2.0)
    p = _projector(vols)
    try:
        ref1 = _np(p.project_tensors(*projs, area_density=True))
        ref2 = _np(p.project_tensors(*other, area_density=True))
        g = p.capture(*projs, area_density=True)
        out = _np(g.launch())
        for k in ref1:
            np.testing.assert_array_equal(out[k], ref1[k])
        g.set_views(*other)
        out = _np(g.launch())
        for k in ref2:
            np.testing.assert_array_equal(out[k], ref2[k])
        out = _np(g.launch())  # replays keep giving the same images
        np.testing.assert_array_equal(out["intensity"], ref2["intensity"])
        with pytest.raises(ValueError):
            g.set_views(*other[:3])
        g.close()
    finally:
        p.free()


def test_autotune_returns_a_valid_shape(tmp_path, monkeypatch):
    monkeypatch.setenv("DEEPDRR_GB300_CACHE", str(tmp_path))
    vols, projs = _scene(1, views=4)
    p = _projector(vols)
    try:
        best = p.autotune(*projs)
        assert best["tile_warps_x"] in (1, 2, 4) and best["blocks_per_sm"] >= 1 and best["items_per_grab"] >= 1
        assert best["ms_per_view"] > 0
        assert p.autotune(*projs) == best  # served from the cache file
        plain = _np(p.project_tensors(*projs))
        tuned = _np(p.project_tensors(*projs, persistent=True, launch=best))
        np.testing.assert_array_equal(plain["intensity"], tuned["intensity"])
    finally:
        p.free()
