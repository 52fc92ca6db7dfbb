"""The multi-volume march follows the shared label-cache key only inside an alpha range per ray
(deepdrr_gb300/csrc/drr_coincide.h). That range must hold every step where two volumes' bases
coincide: checked here against a brute-force float32 march over random geometries, many of them
built to coincide (shared or nearly shared voxel grids)."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("coincide") / "libcoincide.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                           str(HERE / "coincide_shim.cpp"), "-o", str(out)])
    lib = ctypes.CDLL(str(out))
    lib.check_range.restype = ctypes.c_int
    lib.check_range.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_float,
                                ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    return lib


def _rotation(rng, deg):
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    th = np.deg2rad(deg)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


@pytest.mark.parametrize("trials, reach, alpha_max, seed", [(400, 300.0, 2.0, 0), (1500, 2000.0, 3000.0, 123)])
def test_range_holds_every_coincidence(shim, trials, reach, alpha_max, seed):
    """Sources up to `reach` voxels from the grids' origins and marches starting at alpha up to
    `alpha_max` (then 6000 steps): the float32 range's rounding grows with |s| and |alpha r|."""
    rng = np.random.default_rng(seed)
    total_seen = 0
    for trial in range(trials):
        nv = int(rng.integers(2, 5))
        ray = rng.normal(size=3)
        ray /= np.linalg.norm(ray)
        src = rng.uniform(-reach, reach, 3)
        s, r = [], []
        base_A = np.diag(1.0 / rng.uniform(0.5, 1.5, 3)) @ _rotation(rng, rng.uniform(0, 180))
        base_o = rng.uniform(0, 100, 3)
        for i in range(nv):
            kind = rng.integers(0, 3)
            if kind == 0:  # the same voxel grid as volume 0
                A, o = base_A, base_o
            elif kind == 1:  # a nearly identical grid
                A = base_A @ _rotation(rng, rng.uniform(0, 0.5))
                o = base_o + rng.uniform(-1.5, 1.5, 3)
            else:  # unrelated
                A = np.diag(1.0 / rng.uniform(0.3, 2.0, 3)) @ _rotation(rng, rng.uniform(0, 180))
                o = rng.uniform(-50, 150, 3)
            ri = (A @ ray).astype(np.float32)
            si = (A @ src + o).astype(np.float32)
            s.append(si)
            r.append(ri)
        s = np.ascontiguousarray(np.array(s, dtype=np.float32))
        r = np.ascontiguousarray(np.array(r, dtype=np.float32))
        step = float(rng.choice([0.1, 0.25, 0.05, 1.0]))
        seen = ctypes.c_int(0)
        outside = shim.check_range(nv, s.ctypes.data, r.ctypes.data, step, float(rng.uniform(0.5, alpha_max)), 6000,
                                   ctypes.byref(seen))
        total_seen += seen.value
        assert outside == 0, (trial, nv, step, seen.value)
    assert total_seen > 1000  # the geometries above do produce coincidences
