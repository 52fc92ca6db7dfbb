"""Golden vectors of the reference's detector noise, deepdrr/projector/analytic_generators.py:10-18.

The reference's ``add_noise`` draws its variates from numpy's global generator, which no GPU
generator reproduces. What can be pinned is everything around the variates: this script runs the
reference's own function with ``np.random.poisson`` returning given counts (and ``np.random.randn``
zeros, which the reference scales by factor_electronic_noise = 0 anyway) and records inputs, counts
and outputs. The counts are this library's own Poisson variates: its Philox4x32-10 + inversion /
PTRS sampler (deepdrr_gb300/csrc/drr_philox.h) compiled for the host through tests/philox_shim.cpp.
tests/test_noise_cpu.py then holds oracle/noise.py (which the GPU tests hold drr_add_noise to) to
these outputs.

Run where the DeepDRR sources are available (``--reference``, default: the DEEPDRR_REFERENCE
environment variable, as oracle/build_ref.py resolves it):

    python tests/golden/make_noise_vectors.py [--reference PATH] [--out tests/golden/noise_reference.npz]
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle.build_ref import default_reference  # noqa: E402

PHOTON_COUNT = 10000  # Projector(photon_count=...) default, projector.py:398-422
SEED = 2024


def library_counts(lam: np.ndarray, seed: int) -> np.ndarray:
    """The library's Poisson variates for lambda (flat index = counter), as drr_poisson_sample draws them."""
    with tempfile.TemporaryDirectory() as d:
        so = Path(d) / "libphilox.so"
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(ROOT / "tests" / "philox_shim.cpp"),
                               "-o", str(so)])
        lib = ctypes.CDLL(str(so))
        lib.poisson_many.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_ulonglong, ctypes.c_void_p]
        flat = np.ascontiguousarray(lam, dtype=np.float32).ravel()
        out = np.empty_like(flat)
        lib.poisson_many(flat.ctypes.data, flat.size, seed, out.ctypes.data)
    return out.reshape(lam.shape)


def load_reference_module(reference: Path):
    path = reference / "deepdrr" / "projector" / "analytic_generators.py"
    spec = importlib.util.spec_from_file_location("_ref_analytic_generators", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    import scipy.signal  # noqa: F401  (the module calls scipy.signal.convolve2d through `import scipy`)
    return mod


def inputs(rng):
    """Three [40, 52] float32 views: intensities and photon probabilities as a projector makes them
    (probabilities in (0, 1]), with one pixel of photon_prob 0 (lambda 0: the reference's 0/0)."""
    n, h, w = 3, 40, 52
    prob = rng.uniform(1e-4, 1.0, (n, h, w)).astype(np.float32)
    prob[1, 17, 23] = 0.0
    inten = (prob * rng.uniform(20.0, 60.0, (n, h, w))).astype(np.float32)
    return inten, prob


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(default_reference()))
    ap.add_argument("--out", default=str(Path(__file__).with_name("noise_reference.npz")))
    args = ap.parse_args()
    ref = load_reference_module(Path(args.reference))
    inten, prob = inputs(np.random.default_rng(11))
    lam = prob * np.float32(PHOTON_COUNT)  # float32, as numpy computes photon_prob * photon_number
    counts = library_counts(lam, SEED)
    queue = [counts[i] for i in range(counts.shape[0])]
    poisson, randn = np.random.poisson, np.random.randn
    np.random.poisson = lambda lam_i: queue.pop(0).astype(np.int64)
    np.random.randn = lambda *shape: np.zeros(shape)
    try:
        with np.errstate(divide="ignore", invalid="ignore"):
            out = ref.add_noise(inten, prob, PHOTON_COUNT)
    finally:
        np.random.poisson, np.random.randn = poisson, randn
    np.savez_compressed(args.out, intensity=inten, photon_prob=prob, counts=counts, photon_count=PHOTON_COUNT,
                        seed=SEED, output=out)
    print(f"wrote {args.out}: output {out.shape} {out.dtype}, NaN pixels {int(np.isnan(out).sum())}")


if __name__ == "__main__":
    main()
