"""GPU tests of the additive mesh path (drr_mesh_area_density and its use in drr_project) against
the oracle's restatement of the reference's density pass (oracle/mesh.py).

Tolerances: the same pixels covered (exact integer coverage); integrals within 1e-6 relative
(+1e-5 mm g/cm^3: float64 sums in a different order, rounded to float32). In the projector, the mesh
material's path length moves by the integral / 10 (float32 addition before the division) and no
other material's changes at all.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import ctypes

import deepdrr_gb300 as dd
from deepdrr_gb300 import _lib, geo, tables
from deepdrr_gb300.mesh import Mesh
from deepdrr_gb300.phantoms import random_views, simple_phantom_hu, volume_from_hu
from oracle.mesh import mesh_area_density

from helpers import GOLDEN_TABLES

pytestmark = pytest.mark.gpu


def gpu_mesh(meshes, projs, n_slots, slot_of):
    tri = np.concatenate([m.triangles_in_world().reshape(-1, 9) for m in meshes]).astype(np.float32)
    slot = np.concatenate([np.full(len(m.faces), slot_of[m.material], np.int32) for m in meshes])
    dens = np.concatenate([np.full(len(m.faces), m.density, np.float32) for m in meshes])
    views = [geo.view_arrays(p) for p in projs]
    w, h = views[0][2], views[0][3]
    wfi = np.ascontiguousarray(np.stack([v[0] for v in views]), dtype=np.float64)
    src = np.ascontiguousarray(np.stack([v[1] for v in views]), dtype=np.float64)
    t = [torch.from_numpy(x).cuda() for x in (tri, slot, dens)]
    out = torch.empty((len(projs), n_slots, h, w), dtype=torch.float32, device="cuda")
    d = _lib.drr_mesh_desc(triangles=t[0].data_ptr(), slot=t[1].data_ptr(), density=t[2].data_ptr(),
                           n_triangles=len(tri), n_slots=n_slots)
    _lib.check(_lib.load().drr_mesh_area_density(ctypes.byref(d), w, h, len(projs), wfi.ctypes.data, src.ctypes.data,
                                                 None, None, 0, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu().numpy(), (tri, slot, dens, wfi, src, w, h)


def test_rasterizer_matches_the_oracle():
    meshes = [Mesh.icosphere(9.0, center=(2.0, -1.0, 3.0), subdivisions=3, material="titanium"),
              Mesh.box((6.0, 14.0, 5.0), center=(-4.0, 3.0, -2.0), material="iron")]
    slot_of = {"iron": 0, "titanium": 1}
    projs = random_views(3, np.zeros(3), seed=3, sphere_mm=3.0, cone_deg=70.0, sensor_size=(72, 56), pixel_size=0.9,
                         fraction_range=(0.5, 0.6))
    got, (tri, slot, dens, wfi, src, w, h) = gpu_mesh(meshes, projs, 2, slot_of)
    for k in range(len(projs)):
        ref = mesh_area_density(tri, slot, dens, 2, wfi[k], src[k], w, h)
        assert np.array_equal(got[k] > 0, ref > 0), k
        np.testing.assert_allclose(got[k], ref, rtol=1e-6, atol=1e-5)
        assert (ref[1] > 0).sum() > 100 and (ref[0] > 0).sum() > 100


def test_projector_adds_the_mesh_to_its_material_only():
    vol = volume_from_hu(simple_phantom_hu(40, seed=2))
    mesh = Mesh.icosphere(6.0, center=vol.center_in_world + np.array([3.0, 0.0, 2.0]), material="titanium")
    projs = random_views(2, vol.center_in_world, seed=5, sphere_mm=2.0, sensor_size=(48, 40), pixel_size=2.0,
                         fraction_range=(0.5, 0.6))
    src = tables.NpzTables(GOLDEN_TABLES)
    kw = dict(spectrum="90KV_AL40", tables=src, neglog=False, step=0.1)
    with dd.Projector([vol, mesh], **kw) as p:
        mats = p.all_materials
        with_mesh = p.project_tensors(*projs, area_density=True)
        persistent = p.project_tensors(*projs, area_density=True, persistent=True)
        g = p.capture(*projs, area_density=True)
        graphed = {k: v.clone() for k, v in g.launch().items()}
        g.close()
    assert "titanium" in mats
    mesh.enabled = False
    with dd.Projector([vol, mesh], **kw) as p:
        without = p.project_tensors(*projs, area_density=True)
    ti = mats.index("titanium")
    tri = mesh.triangles_in_world().reshape(-1, 9)
    for k, proj in enumerate(projs):
        W, s, w, h = geo.view_arrays(proj)
        add = mesh_area_density(tri, np.zeros(len(tri), np.int32), np.full(len(tri), mesh.density, np.float32), 1,
                                W, s, w, h)[0]
        a1 = with_mesh["area_density"][k].cpu().numpy()
        a0 = without["area_density"][k].cpu().numpy()
        for m in range(len(mats)):
            if m != ti:
                np.testing.assert_array_equal(a1[m], a0[m])
        # the kernel adds the integral to the step-scaled sum before dividing by 10
        np.testing.assert_allclose(a1[ti] - a0[ti], add / 10.0, rtol=1e-5, atol=2e-6)
        assert (add > 0).sum() > 50
    for k in ("intensity", "photon_prob", "area_density"):
        assert torch.equal(with_mesh[k], persistent[k]), k
        assert torch.equal(with_mesh[k], graphed[k]), k


def test_subtractive_hit_lists_and_layer_subtraction_match_the_oracle():
    """A layer-1 subtractive sphere inside a layer-0 additive box: the hit lists (sorted crossings)
    and the box's integral with the sphere's part removed, against the oracle."""
    from oracle.mesh import hit_lists

    box = Mesh.box((20.0, 16.0, 18.0), material="iron")
    hole = Mesh.icosphere(6.0, center=(1.0, 0.5, -1.0), subdivisions=2, material="iron", additive=False,
                          subtractive=True, layer=1)
    meshes = [box, hole]
    tri = np.concatenate([m.triangles_in_world().reshape(-1, 9) for m in meshes]).astype(np.float32)
    slot = np.zeros(len(tri), np.int32)
    dens = np.full(len(tri), 7.87, np.float32)
    layer = np.concatenate([np.full(len(m.faces), m.layer, np.int32) for m in meshes])
    mode = np.concatenate([np.full(len(m.faces), (1 if m.additive else 0) | (2 if m.subtractive else 0), np.uint8)
                           for m in meshes])
    proj = random_views(1, np.zeros(3), seed=8, sphere_mm=1.0, cone_deg=40.0, sensor_size=(56, 48), pixel_size=1.0,
                        fraction_range=(0.5, 0.5))[0]
    W, s, w, h = geo.view_arrays(proj)
    wfi = np.ascontiguousarray(W, dtype=np.float64)
    src = np.ascontiguousarray(s, dtype=np.float64)
    L, K = 2, 8
    t = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (tri, slot, dens, layer, mode)]
    d = _lib.drr_mesh_desc(triangles=t[0].data_ptr(), slot=t[1].data_ptr(), density=t[2].data_ptr(),
                           layer=t[3].data_ptr(), mode=t[4].data_ptr(), n_triangles=len(tri), n_slots=1, n_layers=L)
    ha = torch.empty((L, h, w, K), dtype=torch.float32, device="cuda")
    hf = torch.empty((L, h, w, K), dtype=torch.int8, device="cuda")
    lib = _lib.load()
    _lib.check(lib.drr_mesh_hits(ctypes.byref(d), w, h, wfi.ctypes.data, src.ctypes.data, K, ha.data_ptr(),
                                 hf.data_ptr(), None))
    out = torch.empty((1, 1, h, w), dtype=torch.float32, device="cuda")
    _lib.check(lib.drr_mesh_area_density(ctypes.byref(d), w, h, 1, wfi.ctypes.data, src.ctypes.data, ha.data_ptr(),
                                         hf.data_ptr(), K, out.data_ptr(), None))
    torch.cuda.synchronize()
    A, F = hit_lists(tri, layer, mode, L, K, W, s, w, h)
    np.testing.assert_array_equal(hf.cpu().numpy(), F)
    np.testing.assert_allclose(ha.cpu().numpy(), A, rtol=1e-6, atol=1e-4)
    assert (F[1, :, :, 0] == 1).sum() > 50 and (F[0] == 0).all()
    ref = mesh_area_density(tri, slot, dens, 1, W, s, w, h, layer=layer, mode=mode, hits=(A, F))
    got = out.cpu().numpy()[0]
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-3)
    plain = mesh_area_density(tri, slot, dens, 1, W, s, w, h, layer=layer, mode=mode)
    carved = F[1, :, :, 0] == 1
    assert np.all(ref[0][carved] < plain[0][carved])


def test_subtractive_mesh_carves_the_volume():
    """A subtractive box inside a uniform cube: along the axis the cube's material loses the box's
    chord (to within the two boundary samples), and nothing changes elsewhere."""
    from helpers import uniform_cube

    vol = uniform_cube(40, density=1.0, spacing=1.0, material="soft tissue")
    hole = Mesh.box((10.0, 10.0, 8.0), material="air", additive=False, subtractive=True, layer=0)
    proj = geo.CameraProjection.from_view((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), up=(0.0, -1.0, 0.0),
                                          source_to_detector_distance=1000.0, pixel_size=1.0, sensor_size=(32, 32),
                                          source_to_point_fraction=0.5)
    src = tables.NpzTables(GOLDEN_TABLES)
    kw = dict(spectrum="90KV_AL40", tables=src, neglog=False, step=0.1)
    with dd.Projector([vol, hole], **kw) as p:
        carved = p.project_tensors(proj, area_density=True)["area_density"][0].cpu().numpy()
        st = p.all_materials.index("soft tissue")
    hole.enabled = False
    with dd.Projector([vol, hole], **kw) as p:
        full = p.project_tensors(proj, area_density=True)["area_density"][0].cpu().numpy()
    diff = (full[st] - carved[st]) * 10.0  # mm g/cm^3 removed
    # centre pixels cross the 8 mm box along its depth (magnification 2: the box spans ~20 pixels)
    assert abs(diff[16, 16] - 8.0) <= 0.25
    assert np.all(np.abs(diff[:4]) < 1e-6) and np.all(np.abs(diff[:, :4]) < 1e-6)


# ---------------------------------------------------------------- against the reference kernel --

def _mesh_buffers(p, proj):
    """The projector's own rasterisation for one view: subtractive hit lists [L][H][W][K] and the
    per-slot additive integrals [S][H][W] (what drr_project reads), with the slots' materials."""
    keep = []
    desc = p._mesh_desc(keep)
    W, s, w, h = geo.view_arrays(proj)
    wfi = np.ascontiguousarray(W[None], dtype=np.float64)
    src = np.ascontiguousarray(np.asarray(s)[None], dtype=np.float64)
    L, K = p.mesh_layers, p.max_mesh_hits
    ha = torch.empty((L, h, w, K), dtype=torch.float32, device="cuda")
    hf = torch.empty((L, h, w, K), dtype=torch.int8, device="cuda")
    lib = _lib.load()
    _lib.check(lib.drr_mesh_hits(ctypes.byref(desc), w, h, wfi.ctypes.data, src.ctypes.data, K, ha.data_ptr(),
                                 hf.data_ptr(), None))
    S = len(p.mesh_materials)
    out = torch.empty((1, S, h, w), dtype=torch.float32, device="cuda")
    p._mesh_fill(desc, wfi, src, w, h, out, (ha, hf))
    torch.cuda.synchronize()
    mats = np.asarray([p.all_materials.index(m) for m in p.mesh_materials], dtype=np.int32)
    return ha.cpu().numpy(), hf.cpu().numpy(), out[0].cpu().numpy(), mats


def test_forward_consumes_meshes_like_the_reference_kernel():
    """The march's use of subtractive hit lists (project_kernel.cu:498-521: a sample inside any
    layer adds nothing) and of additive integrals (project_kernel.cu:569-579: added per material
    after the step scaling, before the division by 10), against the reference kernel compiled with
    MESH_ADDITIVE_ENABLED=1 and given the same hit lists and integrals in its own layouts
    ([2][H][W][32] hits with every layer valid; [2][n_mesh_materials][H][W][2] integrals, layer 0
    holding ours with a balanced crossing count). Intensity within 1e-4, path lengths within 1e-5
    relative (read out through one-bin spectra) plus read-out noise."""
    from oracle import ref_kernel

    from helpers import DeltaTables, labels_for

    vol = volume_from_hu(simple_phantom_hu(40, seed=2))
    c = vol.center_in_world
    tool = Mesh.icosphere(6.0, center=c + np.array([3.0, 0.0, 2.0]), material="titanium")
    cut = Mesh.box((12.0, 9.0, 10.0), center=c + np.array([-4.0, 1.0, -1.0]), material="titanium", additive=False,
                   subtractive=True, layer=0)
    cut2 = Mesh.icosphere(4.0, center=c + np.array([5.0, -3.0, 0.0]), subdivisions=2, material="titanium",
                          additive=False, subtractive=True, layer=1)
    proj = random_views(1, c, seed=9, sphere_mm=2.0, sensor_size=(48, 40), pixel_size=2.0,
                        fraction_range=(0.5, 0.6))[0]
    golden = tables.NpzTables(GOLDEN_TABLES)
    W, s, w, h = geo.view_arrays(proj)
    with dd.Projector([vol, tool, cut, cut2], spectrum="90KV_AL40", tables=golden, neglog=False, step=0.1) as p:
        mats = p.all_materials
        if not ref_kernel.available(1, len(mats), mesh_additive=True):
            pytest.skip("reference cubins not built (no reference sources where this tree was built)")
        assert p.mesh_layers == ref_kernel.MESH_LAYERS and p.max_mesh_hits == ref_kernel.MAX_MESH_HITS
        ha, hf, add, slot_mats = _mesh_buffers(p, proj)
    assert (hf[0] != 0).any() and (hf[1] != 0).any() and (add > 0).sum() > 50
    additive = np.zeros((ref_kernel.MESH_LAYERS, len(slot_mats), h, w, 2), np.float32)
    additive[0, :, :, :, 0] = add
    vols_ref = [dict(density=vol.data, labels=labels_for(vol, mats), ijk_from_world=vol.ijk_from_world.data)]
    for spectrum, src, m in [("90KV_AL40", golden, None)] + [(DeltaTables.SPECTRUM, DeltaTables(n), i)
                                                             for i, n in enumerate(mats)]:
        with dd.Projector([vol, tool, cut, cut2], spectrum=spectrum, tables=src, neglog=False, step=0.1) as p:
            got = {k: v[0].cpu().numpy() for k, v in p.project_tensors(proj, area_density=True).items()}
        e, pdf, mu = tables.build_tables(spectrum, mats, src)
        rs = ref_kernel.RefScene(vols_ref, energies=e, pdf=pdf, mu=mu, mesh_additive=True)
        ref = rs.project(W, s, w, h, step=0.1, hit_alpha=ha, hit_facing=hf, layer_valid=np.ones(2, np.int8),
                         additive=additive, unique_materials=slot_mats)
        rs.close()
        if m is None:
            rel = np.abs(got["intensity"].astype(np.float64) - ref["intensity"]) / ref["intensity"]
            print(f"meshes: intensity max rel {rel.max():.3g}")
            assert rel.max() <= 1e-4
        else:
            pp32 = ref["photon_prob"]
            ad_ref = -np.log(pp32.astype(np.float64))
            noise = 2.0 * np.spacing(pp32).astype(np.float64) / pp32
            err = np.abs(got["area_density"][m].astype(np.float64) - ad_ref)
            print(f"meshes: path length of {mats[m]}: max abs err {err.max():.3g} (max {ad_ref.max():.4g} g/cm^2)")
            assert np.all(err <= 1e-5 * ad_ref + noise), (mats[m], err.max())
