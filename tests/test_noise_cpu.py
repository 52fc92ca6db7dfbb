"""The noise model's random numbers (deepdrr_gb300/csrc/drr_philox.h) on the host: Philox4x32-10
against the published known-answer vectors of its authors, and the Poisson sampler's
distribution against the Poisson law."""
import ctypes
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("philox") / "libphilox.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(HERE / "philox_shim.cpp"), "-o",
                           str(out)])
    lib = ctypes.CDLL(str(out))
    u32p = ctypes.POINTER(ctypes.c_uint32)
    lib.philox.argtypes = [u32p, u32p, u32p]
    lib.poisson_many.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_void_p]
    return lib


# Random123 known-answer vectors for philox4x32-10: (counter, key) -> output
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(shim, ctr, key, want):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    shim.philox(c, k, o)
    assert tuple(o) == want


def _sample(shim, lam, n, seed=1234):
    lam_arr = np.full(n, lam, dtype=np.float32)
    out = np.empty(n, dtype=np.float32)
    shim.poisson_many(lam_arr.ctypes.data, n, seed, out.ctypes.data)
    return out


def _pmf(k, lam):
    return np.exp(k * math.log(lam) - lam - np.array([math.lgamma(x + 1) for x in k]))


@pytest.mark.parametrize("lam", [0.3, 2.5, 9.9, 10.0, 37.0, 1000.0, 25000.0])
def test_poisson_distribution(shim, lam):
    """Mean and variance within 5 standard errors, and a chi-square test over the central bins."""
    n = 200000
    x = _sample(shim, lam, n).astype(np.float64)
    assert np.all(x == np.round(x)) and x.min() >= 0
    se_mean = math.sqrt(lam / n)
    assert abs(x.mean() - lam) <= 5 * se_mean
    # variance of the sample variance of a Poisson law: (lam + 2 lam^2 (n/(n-1))) / n ~ (lam + 2 lam^2) / n
    se_var = math.sqrt((lam + 2 * lam * lam) / n)
    assert abs(x.var() - lam) <= 5 * se_var
    lo = max(0, int(lam - 4 * math.sqrt(lam)))
    hi = int(lam + 4 * math.sqrt(lam)) + 2
    ks = np.arange(lo, hi)
    expected = n * _pmf(ks, lam)
    keep = expected >= 20
    ks, expected = ks[keep], expected[keep]
    observed = np.array([(x == k).sum() for k in ks], dtype=np.float64)
    chi2 = float(((observed - expected) ** 2 / expected).sum())
    dof = len(ks)
    # 5-sigma upper bound of a chi-square with dof degrees of freedom
    assert chi2 <= dof + 5 * math.sqrt(2 * dof), (chi2, dof)


def test_poisson_edge_values(shim):
    lam = np.array([0.0, -1.0, np.nan, np.inf, 1e-30], dtype=np.float32)
    out = np.empty(5, dtype=np.float32)
    shim.poisson_many(lam.ctypes.data, 5, 7, out.ctypes.data)
    assert out[0] == 0.0 and np.isnan(out[1]) and np.isnan(out[2]) and np.isnan(out[3]) and out[4] == 0.0


def test_streams_are_independent_of_order(shim):
    """A variate depends only on (seed, index): element i is the same in any batch."""
    lam = np.linspace(0.1, 500.0, 1000).astype(np.float32)
    a = np.empty_like(lam)
    shim.poisson_many(lam.ctypes.data, lam.size, 99, a.ctypes.data)
    b = np.empty(10, dtype=np.float32)
    shim.poisson_many(lam.ctypes.data, 10, 99, b.ctypes.data)
    np.testing.assert_array_equal(a[:10], b)
    c = np.empty_like(lam)
    shim.poisson_many(lam.ctypes.data, lam.size, 100, c.ctypes.data)
    assert np.mean(a == c) < 0.5


# ---- the deterministic part of the noise step, pinned to the reference's own add_noise ----------

GOLDEN_NOISE = HERE / "golden" / "noise_reference.npz"


def test_noise_restatement_matches_the_reference_given_the_same_variates():
    """oracle/noise.py (which the GPU tests hold drr_add_noise to) against the reference's
    add_noise (analytic_generators.py:10-18) run on the same inputs with np.random.poisson returning
    the library's variates (tests/golden/make_noise_vectors.py): bit for bit, NaN pattern included."""
    from oracle.noise import add_noise_given_counts

    g = np.load(GOLDEN_NOISE)
    got = add_noise_given_counts(g["intensity"], g["photon_prob"], g["counts"], float(g["photon_count"]))
    np.testing.assert_array_equal(np.isnan(got), np.isnan(g["output"]))
    assert np.isnan(g["output"]).sum() == 9  # the 3x3 neighbourhood of the photon_prob = 0 pixel
    np.testing.assert_array_equal(got, g["output"])


def test_noise_fixture_holds_the_library_variates(shim):
    """The fixture's counts are what the library's sampler draws for its lambdas under its seed."""
    g = np.load(GOLDEN_NOISE)
    lam = (g["photon_prob"] * np.float32(g["photon_count"])).astype(np.float32).ravel()
    out = np.empty_like(lam)
    shim.poisson_many(lam.ctypes.data, lam.size, int(g["seed"]), out.ctypes.data)
    np.testing.assert_array_equal(out.reshape(g["counts"].shape), g["counts"])


def test_noise_fixture_reproduces_with_the_reference_sources():
    """Where the reference sources are present, its add_noise run again gives the recorded output."""
    from oracle.build_ref import default_reference

    ref = default_reference()
    if not (ref / "deepdrr" / "projector" / "analytic_generators.py").is_file():
        pytest.skip("needs the DeepDRR sources")
    import sys

    sys.path.insert(0, str(HERE / "golden"))
    try:
        import make_noise_vectors as mk
    finally:
        sys.path.pop(0)
    mod = mk.load_reference_module(ref)
    g = np.load(GOLDEN_NOISE)
    queue = [g["counts"][i] for i in range(g["counts"].shape[0])]
    poisson, randn = np.random.poisson, np.random.randn
    np.random.poisson = lambda lam_i: queue.pop(0).astype(np.int64)
    np.random.randn = lambda *shape: np.zeros(shape)
    try:
        with np.errstate(divide="ignore", invalid="ignore"):
            out = mod.add_noise(g["intensity"], g["photon_prob"], int(g["photon_count"]))
    finally:
        np.random.poisson, np.random.randn = poisson, randn
    np.testing.assert_array_equal(out, g["output"])
