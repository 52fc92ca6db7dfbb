"""The adjoint's integer form of the texture unit's linear filter (deepdrr_gb300/csrc/drr_texweights.h):
the packed two-lane corner weights against the staged scalar rule for every fraction triple, the
run sums formed from the staged terms against the summed packed weights, and the fused fixed-point
coordinate against the clamp-then-round form on random and edge coordinates."""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("texweights") / "libtexweights.so"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                           str(HERE / "texweights_shim.cpp"), "-o", str(out)])
    lib = ctypes.CDLL(str(out))
    lib.packed_mismatches.restype = ctypes.c_longlong
    lib.term_mismatches.restype = ctypes.c_longlong
    for f in (lib.fix_kernel_form, lib.fix_staged_form):
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_float, ctypes.c_int]
    return lib


def test_packed_weights_match_the_staged_rule_for_every_fraction(shim):
    assert shim.packed_mismatches() == 0


def test_run_sums_from_the_staged_terms_equal_the_summed_packed_weights(shim):
    assert shim.term_mismatches() == 0


def test_fixed_point_coordinate_forms_agree(shim):
    rng = np.random.default_rng(0)
    cases = []
    for n in (1, 2, 28, 256, 400, 512, 4096, 32767):
        xs = np.concatenate([
            rng.uniform(-2.0, n + 1.0, 4000),
            np.arange(-2.0, min(n, 40) + 1.0, 1.0 / 512),  # every half-step boundary near the low face
            n - 0.5 + np.arange(-64, 64) / 1024.0,           # around the high clamp
        ]).astype(np.float32)
        # neighbours of the rounding boundaries (k + 0.5) / 256 + 0.5
        k = rng.integers(-256, 256 * n, 2000)
        b = ((k + 0.5) / 256.0 + 0.5).astype(np.float32)
        xs = np.concatenate([xs, b, np.nextafter(b, np.float32(-np.inf)), np.nextafter(b, np.float32(np.inf))])
        for x in xs:
            cases.append((float(x), n))
    bad = [(x, n) for x, n in cases if shim.fix_kernel_form(x, n) != shim.fix_staged_form(x, n)]
    assert not bad, bad[:10]
