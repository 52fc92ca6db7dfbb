"""CPU tests of the C ABI: the library builds, loads and exports every declared entry point, and
argument validation answers before any CUDA call (so these run without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

from deepdrr_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "drr_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(drr_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_binding_table():
    assert set(declared_functions()) == set(_lib.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.drr_version().decode().startswith("deepdrr-gb300")


def test_invalid_arguments_are_rejected_on_the_host():
    lib = _lib.load()
    out = ctypes.c_void_p()
    assert lib.drr_volset_create(None, 1, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_INVALID_ARGUMENT
    assert "NULL" in lib.drr_last_error().decode()
    descs = (_lib.drr_volume_desc * 1)()
    assert lib.drr_volset_create(descs, 0, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_INVALID_ARGUMENT
    assert lib.drr_volset_create(descs, 5, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_UNSUPPORTED
    assert lib.drr_volset_create(descs, 1, 0, None, ctypes.byref(out)) == _lib.DRR_ERR_INVALID_ARGUMENT
    assert lib.drr_volset_create(descs, 1, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_INVALID_ARGUMENT
    d = descs[0]
    d.density, d.labels, d.ni, d.nj, d.nk = 16, 16, 4, 4, 0
    assert lib.drr_volset_create(descs, 1, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_INVALID_ARGUMENT
    d.nk, d.density_type = 4, 7
    assert lib.drr_volset_create(descs, 1, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_UNSUPPORTED
    # 16384 texels per axis at most: the 3D texture limit, on which the kernels' 32-bit in-plane
    # label-table offsets rely
    d.density_type = 0
    for axis in ("ni", "nj", "nk"):
        setattr(d, axis, 16385)
        assert lib.drr_volset_create(descs, 1, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_UNSUPPORTED
        assert "16384" in lib.drr_last_error().decode()
        setattr(d, axis, 4)
    assert lib.drr_tables_create(None, None, None, 3, 3, None, ctypes.byref(out)) == _lib.DRR_ERR_INVALID_ARGUMENT
    args = _lib.drr_project_args()
    assert lib.drr_project(None, None, ctypes.byref(args), None) == _lib.DRR_ERR_INVALID_ARGUMENT
    assert lib.drr_neglog(None, 2, 16, 0.01, None) == _lib.DRR_ERR_INVALID_ARGUMENT
    assert lib.drr_neglog(None, 0, 16, 0.01, None) == _lib.DRR_OK  # nothing to do
    assert lib.drr_clip_upper(None, 5, 1.0, None) == _lib.DRR_ERR_INVALID_ARGUMENT
    assert lib.drr_volset_destroy(None) == _lib.DRR_OK
    assert lib.drr_tables_destroy(None) == _lib.DRR_OK
