"""X-ray spectra and mass-attenuation tables for the projector.

The projector needs, per spectrum bin, the energy (keV), the normalised weight and mu/rho (cm^2/g)
of every material, laid out ``mu[bin][material]`` (deepdrr/projector/projector.py:1659-1686).

Sources of the numbers:

* ``NpzTables`` -- a ``.npz`` with ``<S>/spectrum``, ``<S>/energies``, ``<S>/pdf`` and
  ``<S>/mu/<material>`` arrays (the layout written by ``tests/golden/make_golden.py``);
* ``DeepDRRDataTables`` -- a DeepDRR source tree: its NIST tables in
  ``deepdrr/material/material_decompositions`` and its spectra in
  ``deepdrr/projector/spectral_data.py``. Interpolation restates deepdrr/material/material.py:80-110
  and log_interp.py:6-31: linear interpolation of log10(mu/rho) against log10(E [MeV]), with the
  first of two equal edge energies moved down by a factor (1 - 1e-9).

The default source comes from ``DEEPDRR_GB300_TABLES`` (an .npz path) or ``DEEPDRR_DATA_DIR`` (a
DeepDRR checkout), or is set with ``set_default_source``.
"""
from __future__ import annotations

import ast
import os
import re
from pathlib import Path
from typing import Dict, List, Optional, Sequence, Tuple, Union

import numpy as np

# Named-material aliases of deepdrr/material/mappings.py:95-101.
NAMED_MATERIALS = {
    "soft tissue": "tissue_soft",
    "iron": "26_Fe_Iron",
    "lead": "82_Pb_Lead",
    "copper": "29_Cu_Copper",
    "titanium": "22_Ti_Titanium",
}


def spectrum_energies_pdf(spectrum: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """(eV, weight) rows -> (float32 keV, float32 weight / sum) as projector.py:1661-1672."""
    s = np.asarray(spectrum, dtype=np.float64)
    if s.ndim != 2 or s.shape[1] != 2:
        raise ValueError(f"spectrum must be an [n_bins, 2] array of (eV, weight), got {s.shape}")
    energies = np.ascontiguousarray(s[:, 0].copy() / 1000, dtype=np.float32)
    pdf = np.ascontiguousarray(s[:, 1] / np.sum(s[:, 1]), dtype=np.float32)
    return energies, pdf


def log_log_interp(x: Union[float, np.ndarray], xp: np.ndarray, fp: np.ndarray) -> np.ndarray:
    """10 ** interp(log10 x; log10 xp, log10 fp) (log_interp.py:6-31)."""
    return np.power(10, np.interp(np.log10(x), np.log10(xp), np.log10(fp)))


class TableSource:
    def spectrum(self, name: str) -> np.ndarray:
        raise NotImplementedError

    def mu_over_rho(self, material: str, energies_kev: np.ndarray, spectrum_name: Optional[str] = None) -> np.ndarray:
        raise NotImplementedError

    def has_material(self, material: str) -> bool:
        raise NotImplementedError


class NpzTables(TableSource):
    """Precomputed tables at the bin energies of named spectra."""

    def __init__(self, path: Union[str, Path]):
        self.path = Path(path)
        with np.load(self.path) as z:
            self._arrays = {k: z[k] for k in z.files}

    def spectrum_names(self) -> List[str]:
        return sorted({k.split("/")[0] for k in self._arrays if k.endswith("/spectrum")})

    def spectrum(self, name: str) -> np.ndarray:
        key = f"{name}/spectrum"
        if key not in self._arrays:
            raise KeyError(f"unrecognized spectrum: {name}")
        return self._arrays[key]

    def has_material(self, material: str) -> bool:
        return any(k.endswith(f"/mu/{material}") for k in self._arrays)

    def mu_over_rho(self, material, energies_kev, spectrum_name=None) -> np.ndarray:
        e = np.asarray(energies_kev, dtype=np.float32)
        names = [spectrum_name] if spectrum_name else self.spectrum_names()
        for s in names:
            ek = f"{s}/energies"
            mk = f"{s}/mu/{material}"
            if ek in self._arrays and mk in self._arrays and np.array_equal(self._arrays[ek], e):
                return self._arrays[mk].astype(np.float32)
        raise ValueError(f"{self.path} has no mu/rho table for material {material!r} at these energies")


class DeepDRRDataTables(TableSource):
    """NIST tables and spectra read from a DeepDRR source tree."""

    def __init__(self, root: Union[str, Path]):
        root = Path(root)
        if (root / "deepdrr").is_dir():
            root = root / "deepdrr"
        self.root = root
        self.material_dir = root / "material" / "material_decompositions"
        self.spectral_path = root / "projector" / "spectral_data.py"
        if not self.material_dir.is_dir():
            raise FileNotFoundError(f"no material_decompositions under {root}")
        self._cache: Dict[str, np.ndarray] = {}
        self._spectra = None

    def _file_for(self, material: str) -> Path:
        name = NAMED_MATERIALS.get(material, material)
        p = self.material_dir / name
        if not p.is_file():
            for f in self.material_dir.iterdir():  # element symbols, e.g. "Ti" -> 22_Ti_Titanium
                parts = f.name.split("_")
                if len(parts) == 3 and parts[1] == material:
                    return f
            raise ValueError(f"Material {material} not found in material database. Please check the material name.")
        return p

    def _table(self, material: str) -> np.ndarray:
        if material not in self._cache:
            rows = []
            for line in self._file_for(material).read_text().splitlines():
                if line.strip() and not line.startswith("_") and not line.startswith("Energy"):
                    rows.append([float(x) for x in line.split()])
            self._cache[material] = np.asarray(rows, dtype=np.float64)
        return self._cache[material]

    def has_material(self, material: str) -> bool:
        try:
            self._file_for(material)
            return True
        except ValueError:
            return False

    def mu_over_rho(self, material, energies_kev, spectrum_name=None) -> np.ndarray:
        tab = self._table(material)
        energies = tab[:, 0].copy()
        for j in range(1, len(energies)):  # material.py:88-92
            if energies[j] == energies[j - 1]:
                energies[j - 1] *= 1 - 1e-9
        out = np.empty(np.shape(energies_kev), dtype=np.float32)
        flat = np.asarray(energies_kev, dtype=np.float32).reshape(-1)
        res = out.reshape(-1)
        for b, e in enumerate(flat):
            # get_coefficients divides the float32 keV scalar by 1000 in float32 and log_interp takes
            # its log10 in float32 before interpolating in float64 (material.py:108-110, log_interp.py:25)
            res[b] = float(log_log_interp(np.float32(e) / np.float32(1000), energies, tab[:, 1]))
        return out

    def spectrum(self, name: str) -> np.ndarray:
        if self._spectra is None:
            self._spectra = parse_spectral_data(self.spectral_path.read_text())
        if name not in self._spectra:
            raise KeyError(f"unrecognized spectrum: {name}")
        return np.asarray(self._spectra[name], dtype=np.float64)


_ARRAY_RE = re.compile(r"^(\w+)\s*=\s*np\.array\(\s*(\[.*?\])\s*\)", re.S | re.M)
_NAME_RE = re.compile(r"'([^']+)'\s*:\s*(\w+)")


def parse_spectral_data(text: str) -> Dict[str, np.ndarray]:
    """The spectra of deepdrr/projector/spectral_data.py, read as data without running the module:
    each ``NAME = np.array([[eV, weight], ...])`` literal (spectral_data.py:7, 99, 251) and the
    ``spectrums = {'60KV_AL35': NAME, ...}`` map (spectral_data.py:463-467). The numbers are parsed
    as Python float literals, which gives the float64 values numpy builds from them."""
    arrays = {m.group(1): np.asarray(ast.literal_eval(m.group(2)), dtype=np.float64)
              for m in _ARRAY_RE.finditer(text)}
    start = text.find("spectrums")
    if start < 0:
        raise ValueError("no `spectrums` map in the spectral data")
    body = text[start:text.index("}", start)]
    out = {}
    for key, var in _NAME_RE.findall(body):
        if var not in arrays:
            raise ValueError(f"spectrum {key!r} names an unknown array {var}")
        out[key] = arrays[var]
    if not out:
        raise ValueError("the `spectrums` map is empty")
    return out


_DEFAULT: Optional[TableSource] = None


def set_default_source(source: Union[TableSource, str, Path, None]) -> None:
    global _DEFAULT
    if source is None or isinstance(source, TableSource):
        _DEFAULT = source
    else:
        p = Path(source)
        _DEFAULT = NpzTables(p) if p.suffix == ".npz" else DeepDRRDataTables(p)


def default_source() -> TableSource:
    global _DEFAULT
    if _DEFAULT is not None:
        return _DEFAULT
    if os.environ.get("DEEPDRR_GB300_TABLES"):
        _DEFAULT = NpzTables(os.environ["DEEPDRR_GB300_TABLES"])
    elif os.environ.get("DEEPDRR_DATA_DIR"):
        _DEFAULT = DeepDRRDataTables(os.environ["DEEPDRR_DATA_DIR"])
    else:
        raise RuntimeError("no spectrum / attenuation table source: set DEEPDRR_GB300_TABLES to a tables .npz, "
                           "DEEPDRR_DATA_DIR to a DeepDRR checkout, or call deepdrr_gb300.tables.set_default_source")
    return _DEFAULT


def configured_source() -> Optional[TableSource]:
    """The default source if one is set or named by the environment, else None (no error)."""
    try:
        return default_source()
    except RuntimeError:
        return None


def build_tables(spectrum: Union[str, np.ndarray], materials: Sequence[str],
                 source: Optional[TableSource] = None) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(energies keV [n], pdf [n], mu [n, M]) float32 for the sorted material list ``materials``."""
    src = source or default_source()
    if isinstance(spectrum, str):
        name = spectrum
        arr = src.spectrum(spectrum)
    elif isinstance(spectrum, np.ndarray):
        name = None
        arr = spectrum
    else:
        raise TypeError(f"unrecognized spectrum type: {type(spectrum)}")
    energies, pdf = spectrum_energies_pdf(arr)
    mu = np.zeros((energies.shape[0], len(materials)), dtype=np.float32)
    for m, mat in enumerate(materials):
        mu[:, m] = src.mu_over_rho(mat, energies, name)
    return energies, pdf, np.ascontiguousarray(mu)
