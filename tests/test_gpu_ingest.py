"""GPU tests of the volume ingest (drr_ingest_hu, Volume.from_hu(device=...)): bit-exact against
the numpy conversion and thresholding of Volume.from_hu (deepdrr/vol/volume.py:281-351,
load_dicom.py:132-143), in the projector's [k][j][i] layout, and identical projections."""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import deepdrr_gb300 as dd
from deepdrr_gb300 import tables
from deepdrr_gb300.ingest import hu_to_density_and_labels
from deepdrr_gb300.phantoms import random_views, simple_phantom_hu
from deepdrr_gb300.volume import format_materials, hu_to_density, segment_thresholds

from helpers import GOLDEN_TABLES

pytestmark = pytest.mark.gpu


def hu_sample(shape, dtype, seed=0):
    rng = np.random.default_rng(seed)
    hu = rng.uniform(-1100, 3000, shape)
    flat = hu.reshape(-1)
    flat[:8] = [-800.0, 350.0, -800.5, 350.5, -900.0, -1000.0, 0.0, 1e4]  # the thresholds and kinks
    if dtype == np.float32:
        flat[8] = np.nan
        flat[9] = np.nextafter(np.float32(-800.0), np.float32(0.0))
    return hu.astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.int16, np.float64])
@pytest.mark.parametrize("shape", [(37, 29, 45), (64, 64, 64), (1, 3, 70)])
def test_ingest_matches_numpy_bit_for_bit(dtype, shape):
    hu = hu_sample(shape, dtype)
    dens, labs = hu_to_density_and_labels(torch.from_numpy(hu).cuda())
    torch.cuda.synchronize()
    want = hu_to_density(hu).astype(np.float32).transpose(2, 1, 0)
    got = dens.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    assert np.array_equal(got[ok].view(np.uint32), want[ok].view(np.uint32))
    _, ids = format_materials(segment_thresholds(hu))
    assert np.array_equal(labs.cpu().numpy(), ids.astype(np.uint8).transpose(2, 1, 0))


@pytest.mark.parametrize("dtype,tdt", [("float16", torch.float16), ("bfloat16", torch.bfloat16)])
def test_ingest_half_storage_rounds_to_nearest(dtype, tdt):
    hu = hu_sample((20, 30, 40), np.float32, seed=3)
    hu[0, 0, 8] = 0.0  # no NaN here
    dens, _ = hu_to_density_and_labels(torch.from_numpy(hu).cuda(), density_dtype=dtype)
    want = torch.from_numpy(hu_to_density(hu).astype(np.float32).transpose(2, 1, 0).copy()).to(tdt)
    assert torch.equal(dens.cpu(), want)


def test_volume_from_hu_on_the_gpu_projects_like_the_host_path():
    hu = simple_phantom_hu(96, seed=5)
    v_host = dd.Volume.from_hu(hu, origin=(-48.0, -48.0, -48.0))
    t0 = time.perf_counter()
    v_host2 = dd.Volume.from_hu(hu, origin=(-48.0, -48.0, -48.0))
    t_host = time.perf_counter() - t0
    v_gpu = dd.Volume.from_hu(torch.from_numpy(hu).cuda(), origin=(-48.0, -48.0, -48.0))
    torch.cuda.synchronize()
    assert np.array_equal(v_host.data.view(np.uint32), v_gpu.data.view(np.uint32))
    assert np.array_equal(v_host.materials[1], v_gpu.materials[1])
    assert v_host.materials[0] == v_gpu.materials[0]
    assert v_gpu.device_arrays(torch.device("cuda", 0)) is not None
    projs = random_views(2, v_host.center_in_world, seed=6, sphere_mm=3.0, sensor_size=(48, 40), pixel_size=3.0,
                         fraction_range=(0.5, 0.6))
    src = tables.NpzTables(GOLDEN_TABLES)
    outs = []
    for v in (v_host, v_gpu):
        with dd.Projector(v, spectrum="90KV_AL40", tables=src, neglog=False) as p:
            outs.append(p.project_tensors(*projs, area_density=True))
    for k in ("intensity", "photon_prob", "area_density"):
        assert torch.equal(outs[0][k], outs[1][k]), k
    print(f"numpy from_hu of 96^3: {t_host * 1e3:.1f} ms")
    # a changed array is not taken from the device copy
    v_gpu.data = v_gpu.data.copy()
    assert v_gpu.device_arrays(torch.device("cuda", 0)) is None
