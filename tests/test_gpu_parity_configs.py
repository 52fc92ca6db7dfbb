"""Parity with the reference's own projectKernel at the benchmark configurations' full sizes.

The small scenes of test_gpu_parity.py march a few hundred steps per ray; a 1536^2 view of the
512 x 512 x 400 CT marches 4,000-6,000, which exercises the float32 `alpha += step` sequence, its
fast-forward and the label-word pipeline far harder. Each test renders one full view with the
product and with the reference kernel (compiled from the reference sources, launched as
_render_single launches it) on identical inputs:

  * C1: 128^3 phantom, 256^2 detector, 120 kVp, 3 materials;
  * C2: 512 x 512 x 400 CT with titanium, 1536^2 detector, 90 kVp, 4 materials;
  * C3: the CT, a 256^3 phantom and a 96 x 96 x 64 titanium implant, each with its own rigid pose,
    384^2 detector, 90 kVp, 4 materials, default priorities.

Tolerances (the projector's specification): intensity and photon_prob within 1e-4 relative;
per-material path lengths within 1e-5 relative, read out of the reference kernel through a one-bin
spectrum (photon_prob = exp(-AD_m) with mu = 1 for material m only) plus the read-out noise of two
float32 ulps of exp(-AD). The measured maxima are printed.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import deepdrr_gb300 as dd
from deepdrr_gb300 import geo, phantoms, tables
from oracle import ref_kernel

from helpers import GOLDEN_TABLES, DeltaTables, labels_for, material_list

pytestmark = pytest.mark.gpu


def product(vols, proj, spectrum, source):
    with dd.Projector(vols, spectrum=spectrum, step=0.1, tables=source, neglog=False) as p:
        out = p.project_tensors(proj, area_density=True)
        torch.cuda.synchronize()
        return {k: v[0].cpu().numpy() for k, v in out.items()}


def reference(vols, proj, spectrum, source):
    mats = material_list(vols)
    e, pdf, mu = tables.build_tables(spectrum, mats, source)
    rs = ref_kernel.RefScene([dict(density=v.data, labels=labels_for(v, mats), ijk_from_world=v.ijk_from_world.data)
                              for v in vols], energies=e, pdf=pdf, mu=mu)
    try:
        W, s, w, h = geo.view_arrays(proj)
        return rs.project(W, s, w, h, step=0.1)
    finally:
        rs.close()


def check_config(name, vols, proj, spectrum):
    mats = material_list(vols)
    if not ref_kernel.available(len(vols), len(mats)):
        pytest.skip("reference cubins not built (no reference sources where this tree was built)")
    src = tables.NpzTables(GOLDEN_TABLES)
    got = product(vols, proj, spectrum, src)
    ref = reference(vols, proj, spectrum, src)
    for k in ("intensity", "photon_prob"):
        rel = np.abs(got[k].astype(np.float64) - ref[k]) / np.abs(ref[k].astype(np.float64))
        print(f"{name}: {k} max rel {rel.max():.3g}, mean {rel.mean():.3g} over {rel.size} rays")
        assert rel.max() <= 1e-4, (k, rel.max())
    for m, mat in enumerate(mats):
        delta = DeltaTables(mat)
        g = product(vols, proj, DeltaTables.SPECTRUM, delta)["area_density"][m].astype(np.float64)
        pp32 = reference(vols, proj, DeltaTables.SPECTRUM, delta)["photon_prob"]
        pp = pp32.astype(np.float64)
        ad_ref = -np.log(pp)
        noise = 2.0 * np.spacing(pp32).astype(np.float64) / pp
        err = np.abs(g - ad_ref)
        crossed = ad_ref > 1e-3
        beyond = np.maximum(err - noise, 0.0)[crossed] / ad_ref[crossed]
        print(f"{name}: path length of {mat}: max rel difference beyond read-out noise "
              f"{beyond.max() if beyond.size else 0:.3g}, max abs {err.max():.3g} g/cm^2, over {crossed.sum()} rays "
              f"crossing it (max {ad_ref.max():.4g} g/cm^2)")
        assert np.all(err <= 1e-5 * ad_ref + noise), (mat, err.max())


def test_c1_full_view_matches_reference_kernel():
    vols, projs, kw = phantoms.workload_simple(seed=0, views=1)
    check_config("C1 128^3 -> 256^2", vols, projs[0], kw["spectrum"])


def test_c2_full_view_matches_reference_kernel():
    vols, projs, kw = phantoms.workload_ct(seed=0, views=1)
    check_config("C2 512x512x400 -> 1536^2", vols, projs[0], kw["spectrum"])


def test_c3_full_view_matches_reference_kernel():
    vols, projs, kw = phantoms.workload_multi(seed=0, views=1)
    check_config("C3 3 volumes -> 384^2", vols, projs[0], kw["spectrum"])
