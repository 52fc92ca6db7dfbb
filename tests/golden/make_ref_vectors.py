"""Golden vectors of the reference's own projectKernel (deepdrr/projector/project_kernel.cu), so that
the CPU test suite can check the oracle against the reference without a GPU.

Run where a GPU is present and ``oracle/_ref`` holds the reference kernel's cubins (compiled from
the reference sources by ``oracle/build_ref.py``):

    python tests/golden/make_ref_vectors.py [OUT.npz]      # default: tests/golden/ref_kernel.npz

It builds five small seeded scenes (one volume at 90 kVp with the solid angle; the same volume
through one-bin spectra that expose each material's path length; two volumes; three volumes, two of
them on one voxel grid, where the reference's shared label cache decides what each reads; one
volume with attenuation outside the volume), runs the reference kernel on every view through
``oracle/ref_harness.cu`` the way ``Projector._render_single`` launches it, and writes each
scene's exact inputs (volumes, float64 matrices, float32 tables) and the kernel's outputs. It
also prints how far the float32 oracle is from the kernel on the same inputs.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

import deepdrr_gb300 as dd  # noqa: E402
from deepdrr_gb300 import geo, tables  # noqa: E402
from deepdrr_gb300.phantoms import implant_volume, random_rigid, random_views, simple_phantom_hu, volume_from_hu  # noqa: E402
from oracle import oracle, ref_kernel  # noqa: E402

from helpers import GOLDEN_TABLES, labels_for, material_list, scene_from_record  # noqa: E402

DELTA_SPECTRUM = np.array([[1000.0, 1.0]])  # one 1 keV bin with pdf 1


def _volume_key(rec, v, labels) -> str:
    """Store a volume (density, remapped labels, pose) once; scenes name it by its key."""
    dens = np.asarray(v.data, np.float32)
    pose = np.asarray(v.ijk_from_world.data, np.float64)
    i = 0
    while f"vol{i}__density" in rec:
        if (np.array_equal(rec[f"vol{i}__density"], dens) and np.array_equal(rec[f"vol{i}__labels"], labels)
                and np.array_equal(rec[f"vol{i}__ijk_from_world"], pose)):
            return f"vol{i}"
        i += 1
    rec[f"vol{i}__density"], rec[f"vol{i}__labels"], rec[f"vol{i}__ijk_from_world"] = dens, labels, pose
    return f"vol{i}"


def _scene_record(shared, name, volumes, projs, *, spectrum, attenuate=False, solid_angle=False, delta_material=None):
    """Inputs of one scene in the form oracle.Scene takes them, plus the reference kernel's outputs."""
    src = tables.NpzTables(GOLDEN_TABLES)
    mats = material_list(volumes, attenuate)
    if delta_material is None:
        e, pdf, mu = tables.build_tables(spectrum, mats, src)
    else:
        e = np.array([1.0], np.float32)
        pdf = np.array([1.0], np.float32)
        mu = np.array([[1.0 if m == delta_material else 0.0 for m in mats]], np.float32)
    rec = dict(shared)
    nv = len(volumes)
    keys = []
    for v in volumes:
        lab = labels_for(v, mats)
        key = _volume_key(rec, v, lab)
        keys.append(key)
    rec[f"{name}__volumes"] = np.array(keys)
    rec[f"{name}__enabled"] = np.array([1 if v.enabled else 0 for v in volumes], np.int32)
    rec[f"{name}__priorities"] = np.array([nv - 1 - i for i in range(nv)], np.int32)
    rec[f"{name}__energies"], rec[f"{name}__pdf"], rec[f"{name}__mu"] = e, pdf, mu
    rec[f"{name}__params"] = np.array([0.1, -4.0, 1.0 if attenuate else 0.0,
                                       float(mats.index("air")) if attenuate else 0.0])  # step, max_ray_length, attenuate, air_index
    ws, ss, outs = [], [], {"intensity": [], "photon_prob": [], "solid_angle": []}
    for proj in projs:
        W, s, w, h = geo.view_arrays(proj)
        ws.append(np.asarray(W, np.float64)[:3, :3])
        ss.append(np.asarray(s, np.float64))
        sc = scene_from_record(rec, name, ws[-1], ss[-1], w, h)
        r = ref_kernel.project(sc, solid_angle=solid_angle)
        for k in outs:
            if k in r:
                outs[k].append(r[k])
        o = sc.project("f32")
        rel = lambda a, b: np.max(np.abs(a.astype(np.float64) - b) / np.abs(b))  # noqa: E731
        print(f"{name}: oracle vs reference kernel, max rel intensity {rel(o['intensity'], r['intensity']):.3g}, "
              f"photon_prob {rel(o['photon_prob'], r['photon_prob']):.3g}")
    rec[f"{name}__world_from_index"] = np.stack(ws)
    rec[f"{name}__source_world"] = np.stack(ss)
    rec[f"{name}__size"] = np.array([w, h], np.int32)
    for k, v in outs.items():
        if v:
            rec[f"{name}__ref_{k}"] = np.stack(v)
    return rec


def main(out: Path) -> None:
    if not ref_kernel.available(1, 3):
        raise SystemExit("reference cubins missing: build them with oracle/build_ref.py first")
    a = volume_from_hu(simple_phantom_hu(32, seed=41))
    views = dict(sphere_mm=3.0, cone_deg=30.0, sensor_size=(24, 20), pixel_size=3.0, fraction_range=(0.5, 0.7))
    projs = random_views(2, a.center_in_world, seed=42, **views)
    rec = {}
    rec = _scene_record(rec, "one", [a], projs, spectrum="90KV_AL40", solid_angle=True)
    for m, mat in enumerate(material_list([a])):
        rec = _scene_record(rec, f"delta{m}", [a], projs, spectrum=DELTA_SPECTRUM, delta_material=mat)

    rng = np.random.default_rng(43)
    b = implant_volume((16, 16, 12), seed=44)
    b.world_from_anatomical = random_rigid(rng, 5.0, 30.0)
    rec = _scene_record(rec, "two", [a, b], projs, spectrum="120KV_AL43")

    names, seg = a.materials
    relabel = {"soft tissue": seg == names["bone"], "bone": seg == names["soft tissue"], "air": seg == names["air"]}
    a2 = dd.Volume.from_parameters(a.data * np.float32(0.7), relabel, origin=-(np.asarray(a.data.shape) - 1) / 2.0,
                                   spacing=(1.0, 1.0, 1.0))
    rec = _scene_record(rec, "three", [a, a2, b], projs, spectrum="90KV_AL40")
    rec = _scene_record(rec, "outside", [a], projs, spectrum="90KV_AL40", attenuate=True)
    out.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out, **rec)
    print(f"wrote {out} ({out.stat().st_size} bytes, {len(rec)} arrays)")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else ROOT / "tests" / "golden" / "ref_kernel.npz")
