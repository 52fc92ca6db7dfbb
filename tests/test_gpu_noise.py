"""GPU tests of the detector noise (drr_add_noise, drr_poisson_sample, Projector(add_noise=True)).

Tolerances: drr_add_noise against the float64 restatement of analytic_generators.add_noise fed the
same variates: 1e-6 relative (+1e-6 absolute), the float32 rounding of the output. Variates against
the host build of the same sampler: equal for at least 99.99 % (device and host libm may differ by
an ulp in exp / log / lgamma at an acceptance boundary); their law: mean and variance within 5
standard errors.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import deepdrr_gb300 as dd
from deepdrr_gb300 import _lib, tables
from deepdrr_gb300.phantoms import random_views, simple_phantom_hu, volume_from_hu
from oracle.noise import add_noise_given_counts

from helpers import GOLDEN_TABLES

pytestmark = pytest.mark.gpu


def poisson_gpu(lam: torch.Tensor, seed: int) -> torch.Tensor:
    out = torch.empty_like(lam)
    _lib.check(_lib.load().drr_poisson_sample(lam.data_ptr(), lam.numel(), seed, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("lam", [0.7, 6.0, 10.0, 150.0, 10000.0])
def test_poisson_law_on_the_gpu(lam):
    n = 1 << 20
    x = poisson_gpu(torch.full((n,), lam, device="cuda"), 17).double()
    assert bool((x == x.round()).all()) and float(x.min()) >= 0
    assert abs(float(x.mean()) - lam) <= 5 * (lam / n) ** 0.5
    assert abs(float(x.var()) - lam) <= 5 * ((lam + 2 * lam * lam) / n) ** 0.5


def test_gpu_variates_match_the_host_build(tmp_path):
    import subprocess
    from pathlib import Path

    here = Path(__file__).resolve().parent
    so = tmp_path / "libphilox.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(here / "philox_shim.cpp"), "-o", str(so)])
    lib = ctypes.CDLL(str(so))
    lib.poisson_many.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_void_p]
    rng = np.random.default_rng(0)
    lam = np.exp(rng.uniform(np.log(0.05), np.log(5e4), 100000)).astype(np.float32)
    host = np.empty_like(lam)
    lib.poisson_many(lam.ctypes.data, lam.size, 4242, host.ctypes.data)
    dev = poisson_gpu(torch.from_numpy(lam).cuda(), 4242).cpu().numpy()
    same = float(np.mean(dev == host))
    print(f"device == host variates: {same:.6f}")
    assert same >= 0.9999


def test_add_noise_matches_the_restatement():
    rng = np.random.default_rng(1)
    n, H, W = 3, 37, 53
    inten = rng.uniform(0.0, 60.0, (n, H, W)).astype(np.float32)
    prob = rng.uniform(0.0, 1.0, (n, H, W)).astype(np.float32)
    prob[0, 5, 7] = 0.0  # a fully attenuated pixel: NaN in its neighbourhood, as in the reference
    N = 10000
    seed = 123456789
    ti, tp = torch.from_numpy(inten).cuda(), torch.from_numpy(prob).cuda()
    out = torch.empty_like(ti)
    _lib.check(_lib.load().drr_add_noise(ti.data_ptr(), tp.data_ptr(), out.data_ptr(), n, H, W, float(N), seed, None))
    lam = (tp * np.float32(N)).contiguous()
    counts = poisson_gpu(lam, seed).cpu().numpy()
    ref = add_noise_given_counts(inten, prob, counts, N)
    got = out.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.isnan(got[0, 4:7, 6:9]).all()
    ok = ~np.isnan(ref)
    np.testing.assert_allclose(got[ok], ref[ok], rtol=1e-6, atol=1e-6)
    assert float(np.abs(got[ok] - inten[ok]).max()) > 0.0


def test_add_noise_rejects_bad_arguments():
    lib = _lib.load()
    t = torch.ones((1, 4, 4), device="cuda")
    assert lib.drr_add_noise(t.data_ptr(), t.data_ptr(), t.data_ptr(), 1, 4, 4, 100.0, 1, None) == \
        _lib.DRR_ERR_INVALID_ARGUMENT
    o = torch.empty_like(t)
    assert lib.drr_add_noise(t.data_ptr(), t.data_ptr(), o.data_ptr(), 1, 4, 4, 0.0, 1, None) == \
        _lib.DRR_ERR_INVALID_ARGUMENT


def test_projector_add_noise_is_seeded_by_numpy_and_unbiased():
    vol = volume_from_hu(simple_phantom_hu(48, seed=2))
    projs = random_views(1, vol.center_in_world, seed=3, sphere_mm=2.0, sensor_size=(40, 32), pixel_size=2.5,
                         fraction_range=(0.5, 0.5))
    src = tables.NpzTables(GOLDEN_TABLES)
    kw = dict(spectrum="90KV_AL40", tables=src, neglog=False)
    with dd.Projector([vol], **kw) as p0:
        clean = p0.project(projs[0]).astype(np.float64)
    with dd.Projector([vol], add_noise=True, photon_count=2000, **kw) as p:
        np.random.seed(5)
        a = p.project(projs[0])
        np.random.seed(5)
        b = p.project(projs[0])
        c = p.project(projs[0])
        np.testing.assert_array_equal(a, b)
        assert not np.array_equal(a, c)
        reps = np.stack([p.project(projs[0]) for _ in range(200)]).astype(np.float64)
    # the noise has zero mean (clipping at 0 is far away here): the average of 200 realisations
    # approaches the clean image within 5 standard errors of that average
    se = reps.std(0) / np.sqrt(reps.shape[0])
    assert np.all(np.abs(reps.mean(0) - clean) <= 5 * se + 1e-6)


# ---------------------------------------------------------------- collected energy --------------

def test_collected_energy_matches_the_restatement():
    """drr_collected_energy (projector.py:833-853 on the GPU) against oracle.collected_energy on the
    same intensities and solid angles: 1e-6 relative (the view's mean solid angle is the correctly
    rounded float32 mean on the GPU and numpy's pairwise float32 mean in the restatement, a few ulps
    apart at most). Also through Projector(collected_energy=True)."""
    from oracle import oracle

    vol = volume_from_hu(simple_phantom_hu(40, seed=3))
    projs = random_views(3, vol.center_in_world, seed=4, sphere_mm=2.0, sensor_size=(70, 52), pixel_size=1.7,
                         fraction_range=(0.5, 0.7))
    src = tables.NpzTables(GOLDEN_TABLES)
    kw = dict(spectrum="90KV_AL40", tables=src, neglog=False, step=0.1)
    with dd.Projector([vol], photon_count=25000, **kw) as p:
        raw = p.project_tensors(*projs, solid_angle=True)
        sdd = p.source_to_detector_distance
    inten, sa = raw["intensity"], raw["solid_angle"]
    area = np.array([(sdd / pr.intrinsic.fx) * (sdd / pr.intrinsic.fy) for pr in projs], dtype=np.float64)
    out = torch.empty_like(inten)
    n, h, w = inten.shape
    _lib.check(_lib.load().drr_collected_energy(inten.data_ptr(), sa.data_ptr(), out.data_ptr(), n, h * w, 25000.0,
                                                area.ctypes.data, None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    I, S = inten.cpu().numpy(), sa.cpu().numpy()
    for i, pr in enumerate(projs):
        ref = oracle.collected_energy(I[i], S[i], 25000, sdd / pr.intrinsic.fx, sdd / pr.intrinsic.fy)
        rel = np.abs(got[i].astype(np.float64) - ref) / np.abs(ref.astype(np.float64))
        assert rel.max() <= 1e-6, rel.max()
    with dd.Projector([vol], photon_count=25000, collected_energy=True, **kw) as p:
        api = p.project(*projs)
    np.testing.assert_array_equal(api, got)
    # in place, and more views than one launch's parameter block holds
    many = inten.repeat(30, 1, 1).contiguous()
    many_sa = sa.repeat(30, 1, 1).contiguous()
    areas = np.tile(area, 30)
    _lib.check(_lib.load().drr_collected_energy(many.data_ptr(), many_sa.data_ptr(), many.data_ptr(), 90, h * w,
                                                25000.0, areas.ctypes.data, None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(many.cpu().numpy(), np.tile(got, (30, 1, 1)))
