"""Spectrum and mass-attenuation tables: the golden fixtures and this package's own restatement of
the reference's log-log interpolation (deepdrr/material/material.py:80-110, log_interp.py:6-31)."""
from pathlib import Path

import numpy as np
import pytest

from deepdrr_gb300 import tables
from oracle.build_ref import default_reference

from helpers import GOLDEN_TABLES

REFERENCE = default_reference()
SPECTRA = ["60KV_AL35", "90KV_AL40", "120KV_AL43"]
MATS = ["air", "soft tissue", "bone", "titanium", "lung", "muscle", "iron", "blood"]


def test_golden_tables_shapes():
    src = tables.NpzTables(GOLDEN_TABLES)
    for s, n in zip(SPECTRA, [91, 151, 211]):
        e, pdf, mu = tables.build_tables(s, ["air", "bone"], src)
        assert e.shape == (n,) and pdf.shape == (n,) and mu.shape == (n, 2)
        assert e.dtype == np.float32 and mu.dtype == np.float32
        assert pdf[-1] < 0  # the last bin of every spectrum has a slightly negative weight
        assert abs(float(pdf.astype(np.float64).sum()) - 1.0) < 1e-5


def test_unknown_spectrum_raises():
    src = tables.NpzTables(GOLDEN_TABLES)
    with pytest.raises(KeyError):
        tables.build_tables("70KV", ["air"], src)
    with pytest.raises(TypeError):
        tables.build_tables(3, ["air"], src)


@pytest.mark.skipif(not REFERENCE.exists(), reason="needs the DeepDRR sources")
def test_own_interpolation_matches_the_reference_bit_for_bit():
    golden = np.load(GOLDEN_TABLES)
    src = tables.DeepDRRDataTables(REFERENCE)
    for s in SPECTRA:
        e, pdf = tables.spectrum_energies_pdf(src.spectrum(s))
        np.testing.assert_array_equal(e, golden[f"{s}/energies"])
        np.testing.assert_array_equal(pdf, golden[f"{s}/pdf"])
        for m in MATS:
            np.testing.assert_array_equal(src.mu_over_rho(m, e), golden[f"{s}/mu/{m}"])
