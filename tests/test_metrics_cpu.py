"""The benchmark's work accounting against the oracle's march.

bench.py reports Gsamples/s with samples counted by ``metrics.count_samples``: a float64 closed form
per ray and volume (slab test, live step range). The oracle counts the same samples one by one while
it marches (project_kernel.cu:472: a volume is sampled at step t when it is traced, enabled and
alpha_t lies in its interval). The closed form must equal the oracle's float64 march. The float32
march (the reference's and the product's) accumulates alpha += step in float32 from about 1 mm in
front of the source, some 5,000 additions of half an ulp (3e-5 mm near alpha = 500 mm) each, so its
interval ends can move by a step or two per ray and volume: about 0.1-0.2 % of the samples here.
bench.py therefore counts the geometry's samples, which the product's march matches to that."""
import numpy as np
import pytest

pytest.importorskip("torch")

from deepdrr_gb300 import metrics
from deepdrr_gb300.phantoms import implant_volume, random_rigid, random_views, simple_phantom_hu, volume_from_hu

from helpers import oracle_scene


def _oracle_samples(vols, proj, mode):
    return oracle_scene(vols, proj).project(mode)["samples"]


@pytest.mark.parametrize("two_volumes", [False, True])
def test_count_samples_matches_the_oracle_march(two_volumes):
    a = volume_from_hu(simple_phantom_hu(40, seed=21))
    vols = [a]
    if two_volumes:
        b = implant_volume((16, 16, 12), seed=22)
        b.world_from_anatomical = random_rigid(np.random.default_rng(23), 5.0, 30.0)
        vols.append(b)
    projs = random_views(3, a.center_in_world, seed=24, sphere_mm=4.0, sensor_size=(24, 20), pixel_size=3.0)
    counted = metrics.count_samples(vols, projs, 0.1, -4.0)
    for i, proj in enumerate(projs):
        s64 = _oracle_samples(vols, proj, "f64")
        s32 = _oracle_samples(vols, proj, "f32")
        print(f"view {i}: closed form {counted[i]:.0f}, oracle float64 {s64:.0f}, float32 {s32:.0f}")
        assert s64 > 1e4
        assert abs(counted[i] - s64) <= 2  # equal here; an interval end within rounding of a step may differ
        rays_x_volumes = 24 * 20 * len(vols)
        assert abs(counted[i] - s32) <= min(2 * rays_x_volumes, 5e-3 * s32)


def test_compulsory_bytes():
    a = volume_from_hu(simple_phantom_hu(8, seed=1))
    assert metrics.compulsory_bytes([a], 4, 2) == 8 ** 3 * 5 + 4 * 2 * 4 * 2
    assert metrics.compulsory_bytes([a], 4, 2, "float16", outputs=1) == 8 ** 3 * 3 + 4 * 2 * 4
