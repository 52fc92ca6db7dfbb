"""CPU tests of the mesh description (deepdrr_gb300.mesh) and of the oracle's restatement of the
additive mesh pass (oracle/mesh.py): winding, STL reading, watertight coverage and path lengths
with known answers."""
import struct

import numpy as np
import pytest

from deepdrr_gb300 import geo
from deepdrr_gb300.mesh import DEFAULT_DENSITIES, Mesh, read_stl
from oracle.mesh import mesh_area_density


def outward(mesh):
    t = mesh.triangles_in_world()
    c = mesh.vertices.mean(0)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    return np.all(np.einsum("ij,ij->i", n, t.mean(1) - c) > 0)


def test_box_and_icosphere_are_wound_outward():
    assert outward(Mesh.box((4.0, 6.0, 8.0), center=(1.0, 2.0, 3.0)))
    assert outward(Mesh.icosphere(5.0, subdivisions=2))


def test_stl_round_trip(tmp_path):
    m = Mesh.icosphere(3.0, subdivisions=1)
    tri = m.triangles_in_world().astype(np.float32)
    p = tmp_path / "s.stl"
    with open(p, "wb") as f:
        f.write(b"\0" * 80 + struct.pack("<I", len(tri)))
        for t in tri:
            f.write(struct.pack("<3f", 0, 0, 0) + t.tobytes() + b"\0\0")
    v, fc = read_stl(p)
    np.testing.assert_array_equal(v[fc].astype(np.float32), tri)
    a = tmp_path / "a.stl"
    lines = ["solid x"]
    for t in tri:
        lines += ["facet normal 0 0 0", "outer loop"] + [f"vertex {float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in t]
        lines += ["endloop", "endfacet"]
    a.write_text("\n".join(lines + ["endsolid x"]))
    v2, f2 = read_stl(a)
    np.testing.assert_allclose(v2[f2], tri, rtol=0, atol=1e-6)
    m2 = Mesh.from_stl(p, material="titanium")
    assert m2.density == DEFAULT_DENSITIES["titanium"] and len(m2.faces) == len(tri)


def test_mesh_flags_and_unknown_density():
    m = Mesh.box(subtractive=True, additive=False, layer=1)
    assert m.subtractive and not m.additive and m.layer == 1
    with pytest.raises(ValueError):
        Mesh.box(additive=False, subtractive=False)
    with pytest.raises(ValueError):
        Mesh.box(material="unobtainium")


def view(direction=(0.0, 0.0, 1.0), sensor=(40, 30), pixel=1.0, sdd=1000.0):
    return geo.CameraProjection.from_view((0.0, 0.0, 0.0), direction, up=(0.0, -1.0, 0.0) if direction[1] == 0 else
                                          (0.0, 0.0, 1.0), source_to_detector_distance=sdd, pixel_size=pixel,
                                          sensor_size=sensor, source_to_point_fraction=0.5)


def oracle_for(mesh, proj, n_slots=1):
    W, s, w, h = geo.view_arrays(proj)
    tri = mesh.triangles_in_world().reshape(-1, 9)
    return mesh_area_density(tri, np.zeros(len(tri), np.int32), np.full(len(tri), mesh.density, np.float32),
                             n_slots, W, s, w, h)


def test_box_path_length_is_exact_through_its_faces():
    """A 10 mm cube seen along z from 500 mm: every covered pixel's ray crosses the front and back
    faces, so the integral is density x chord; near the axis the chord is 10 mm / cos."""
    m = Mesh.box((10.0, 10.0, 10.0), material="iron")
    proj = view()
    out = oracle_for(m, proj)[0]
    W, s, w, h = geo.view_arrays(proj)
    covered = out > 0
    assert covered.sum() > 100
    vv, uu = np.nonzero(covered)
    r = np.stack([uu + 0.5, vv + 0.5, np.ones_like(uu, dtype=float)], 1) @ W.T
    r /= np.linalg.norm(r, axis=1, keepdims=True)
    # rays that cross the z faces (not a side face)
    z0, z1 = -5.0, 5.0
    t0, t1 = (z0 - s[2]) / r[:, 2], (z1 - s[2]) / r[:, 2]
    x0, x1 = s[0] + t0 * r[:, 0], s[0] + t1 * r[:, 0]
    y0, y1 = s[1] + t0 * r[:, 1], s[1] + t1 * r[:, 1]
    through = (np.abs(x0) < 5) & (np.abs(x1) < 5) & (np.abs(y0) < 5) & (np.abs(y1) < 5)
    want = 7.87 * (t1 - t0)
    np.testing.assert_allclose(out[vv[through], uu[through]], want[through], rtol=2e-6)


def test_coverage_is_watertight():
    """Every pixel the sphere covers sees balanced crossings (a ray through a shared edge or vertex
    counts once), so no covered pixel is dropped inside the silhouette."""
    m = Mesh.icosphere(8.0, subdivisions=3, material="titanium")
    proj = view((0.3, 0.2, 1.0), sensor=(64, 64), pixel=0.8)
    W, s, w, h = geo.view_arrays(proj)
    tri = m.triangles_in_world().reshape(-1, 9)
    # unbalanced pixels would be zeroed; compare with the analytic chord of the inscribed sphere
    out = oracle_for(m, proj)[0]
    vv, uu = np.meshgrid(np.arange(h) + 0.5, np.arange(w) + 0.5, indexing="ij")
    r = np.stack([uu, vv, np.ones_like(uu)], -1) @ W.T
    r /= np.linalg.norm(r, axis=-1, keepdims=True)
    b = (r @ -s)
    c2 = b * b - (s @ s - 8.0 ** 2)
    chord = np.where(c2 > 0, 2 * np.sqrt(np.maximum(c2, 0)), 0.0)
    inner = chord > 2.0  # well inside the silhouette
    assert inner.sum() > 200
    assert np.all(out[inner] > 0)
    # the polyhedron is inscribed: its chords are shorter; near the centre by about a percent
    rel = out[inner] / (4.51 * chord[inner])
    assert rel.max() <= 1.0 + 1e-6
    central = chord > 0.95 * 16.0
    assert central.sum() > 10 and (out[central] / (4.51 * chord[central])).min() > 0.97
