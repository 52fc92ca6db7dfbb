"""The kernel's exact fast-forward of `alpha += step` (deepdrr_gb300/csrc/drr_alpha.h) against the
serial float32 loop of the reference (project_kernel.cu:552), on random and boundary cases."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("alpha") / "libalpha.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                           str(HERE / "alpha_shim.cpp"), "-o", str(out)])
    lib = ctypes.CDLL(str(out))
    for f in (lib.fast_forward, lib.serial):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int]
    return lib


def _both(lib, a0, step, bound, limit, inclusive):
    a1 = ctypes.c_float(a0)
    a2 = ctypes.c_float(a0)
    k1 = lib.fast_forward(ctypes.byref(a1), step, bound, limit, inclusive)
    k2 = lib.serial(ctypes.byref(a2), step, bound, limit, inclusive)
    return (k1, np.float32(a1.value)), (k2, np.float32(a2.value))


def test_projector_like_cases(shim):
    """alpha starting at a ray length near 1 mm, step 0.1 mm, bounds at volume entries and exits."""
    rng = np.random.default_rng(0)
    for _ in range(300):
        a0 = float(np.float32(1.0 + rng.uniform(0, 0.2)))
        step = float(np.float32(rng.choice([0.1, 0.05, 0.01, 0.2, 0.025])))
        bound = float(np.float32(rng.uniform(10, 1500)))
        for inclusive in (0, 1):
            ff, se = _both(shim, a0, step, bound, 1 << 26, inclusive)
            assert ff[0] == se[0] and ff[1].tobytes() == se[1].tobytes(), (a0, step, bound, inclusive, ff, se)


def test_random_cases(shim):
    rng = np.random.default_rng(1)
    for _ in range(3000):
        a0 = float(np.float32(rng.choice([0.0, 1e-30, 2.0 ** -10, 1.0, 0.3, 7.0, 255.9, 511.99]) *
                              rng.uniform(0.5, 2.0)))
        step = float(np.float32(10 ** rng.uniform(-5, 1)))
        bound = float(np.float32(a0 + 10 ** rng.uniform(-3, 3)))
        limit = int(rng.integers(0, 200000))
        for inclusive in (0, 1):
            ff, se = _both(shim, a0, step, bound, limit, inclusive)
            assert ff[0] == se[0] and ff[1].tobytes() == se[1].tobytes(), (a0, step, bound, limit, inclusive, ff, se)


def test_ties_and_binade_edges(shim):
    """Steps that are exact half-ulps of alpha, bounds exactly on the float grid, starts at binade tops."""
    for e in range(-3, 10):
        u = 2.0 ** (e - 23)
        for step in (0.5 * u, 1.5 * u, 2.5 * u, 3 * u + 0.5 * u, 0.75 * u, 0.25 * u):
            for a0 in (2.0 ** e, 2.0 ** e + u, 2.0 ** (e + 1) - u, 2.0 ** (e + 1) - 3 * u):
                for bound in (a0 + 1000 * step, 2.0 ** (e + 1), 2.0 ** (e + 2) + 7 * u, float("inf")):
                    for inclusive in (0, 1):
                        ff, se = _both(shim, float(np.float32(a0)), float(np.float32(step)),
                                       float(np.float32(bound)), 50000, inclusive)
                        assert ff[0] == se[0] and ff[1].tobytes() == se[1].tobytes(), (e, step, a0, bound, ff, se)
