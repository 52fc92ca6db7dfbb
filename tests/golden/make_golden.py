"""Generate the golden spectrum / mass-attenuation tables from the reference implementation.

Run where the DeepDRR sources are available (``--reference``, default: the DEEPDRR_REFERENCE
environment variable, as oracle/build_ref.py resolves it):

    python tests/golden/make_golden.py [--reference PATH]

It imports the reference's own ``deepdrr.material`` package and ``deepdrr/projector/spectral_data.py``
(without the top-level ``deepdrr/__init__``, which needs CuPy and an OpenGL stack) and writes
``tests/golden/tables.npz`` with, for every spectrum name of ``spectral_data.spectrums``:

  ``<S>/spectrum``   the raw [n_bins, 2] (eV, weight) array,
  ``<S>/energies``   float32 keV, as ``Projector.initialize`` builds it (projector.py:1661-1664),
  ``<S>/pdf``        float32 w / sum(w) (projector.py:1668-1672),
  ``<S>/mu/<mat>``   float32 mu/rho [cm^2/g] per bin, from
                     ``Material.from_string(mat).get_coefficients(E_keV).mu_over_rho``
                     (projector.py:1676-1686, material.py:80-110, log_interp.py:6-31).

The GPU machines have no copy of the reference, so the tests and the benchmark read these fixtures.
"""
from __future__ import annotations

import argparse
import importlib.util
import sys
import types
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle.build_ref import default_reference  # noqa: E402

MATERIALS = ["air", "soft tissue", "bone", "titanium", "lung", "muscle", "iron", "blood"]


def _load_reference(ref: Path):
    root = ref / "deepdrr"
    pkg = types.ModuleType("deepdrr")
    pkg.__path__ = [str(root)]
    sys.modules["deepdrr"] = pkg
    spec = importlib.util.spec_from_file_location(
        "deepdrr.material", root / "material" / "__init__.py",
        submodule_search_locations=[str(root / "material")])
    mat = importlib.util.module_from_spec(spec)
    sys.modules["deepdrr.material"] = mat
    spec.loader.exec_module(mat)
    spec = importlib.util.spec_from_file_location("_ref_spectral_data", root / "projector" / "spectral_data.py")
    sd = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(sd)
    return mat.Material, sd.spectrums


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(default_reference()))
    ap.add_argument("--out", default=str(Path(__file__).with_name("tables.npz")))
    args = ap.parse_args()
    Material, spectrums = _load_reference(Path(args.reference))
    out = {}
    for name, arr in spectrums.items():
        arr = np.asarray(arr, dtype=np.float64)
        energies = np.ascontiguousarray(arr[:, 0].copy() / 1000, dtype=np.float32)
        pdf = np.ascontiguousarray(arr[:, 1] / np.sum(arr[:, 1]), dtype=np.float32)
        out[f"{name}/spectrum"] = arr
        out[f"{name}/energies"] = energies
        out[f"{name}/pdf"] = pdf
        for m in MATERIALS:
            mu = np.zeros(energies.shape[0], dtype=np.float32)
            for b in range(energies.shape[0]):
                mu[b] = Material.from_string(m).get_coefficients(energies[b]).mu_over_rho
            out[f"{name}/mu/{m}"] = mu
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}: {len(out)} arrays")


if __name__ == "__main__":
    main()
