"""CPU tests of the oracle: analytic known answers, quirks of the reference it restates, and the
texture-filter emulation. No GPU is used."""
import numpy as np
import pytest

from deepdrr_gb300 import geo, tables
from deepdrr_gb300.phantoms import simple_phantom_hu, volume_from_hu, random_views
from oracle import oracle

from helpers import GOLDEN_TABLES, axis_view, oracle_scene, rel_err, uniform_cube


def _center_pixel(scene):
    return scene.sc.height // 2, scene.sc.width // 2


@pytest.mark.parametrize("direction", [(0, 1, 0), (1, 0, 0), (0.3, 1.0, 0.2)])
def test_uniform_cube_path_length_is_the_chord(direction):
    """Area density through a uniform cube = rho x chord (g/cm^2), within one step, for rays
    through the centre (project_kernel.cu:334-584)."""
    n, rho, step = 32, 1.7, 0.1
    vol = uniform_cube(n, rho)
    proj = axis_view(direction, sensor=(8, 8), pixel=0.05)
    sc = oracle_scene([vol], proj, step=step)
    for mode in ("f64", "f32"):
        r = sc.project(mode)
        v, u = _center_pixel(sc)
        ad_cm = float(r["area_density"][0, v, u])
        d = np.asarray(direction, dtype=np.float64)
        d /= np.linalg.norm(d)
        chord = n / np.max(np.abs(d))  # box [-0.5, n-0.5] in mm along the ray through the centre
        assert abs(ad_cm * 10 - rho * chord) <= 2 * step * rho + 1e-3, (mode, ad_cm * 10, rho * chord)


def test_beer_lambert_matches_area_densities():
    """intensity = sum_b E_b pdf_b exp(-sum_m AD_m mu_bm) (project_kernel.cu:637-646)."""
    hu = simple_phantom_hu(48, seed=3)
    vol = volume_from_hu(hu)
    proj = random_views(1, vol.center_in_world, seed=4, sphere_mm=0, sensor_size=(12, 12), pixel_size=4.0)[0]
    sc = oracle_scene([vol], proj, spectrum="90KV_AL40")
    r = sc.project("f64")
    src = tables.NpzTables(GOLDEN_TABLES)
    e, pdf, mu = tables.build_tables("90KV_AL40", ["air", "bone", "soft tissue"], src)
    ad = r["area_density"].reshape(3, -1).T.astype(np.float64)
    x = ad @ mu.T.astype(np.float64)
    p = np.exp(-x) * pdf.astype(np.float64)
    np.testing.assert_allclose(r["photon_prob"].ravel(), p.sum(1), rtol=1e-12)
    np.testing.assert_allclose(r["intensity"].ravel(), (p * e.astype(np.float64)).sum(1), rtol=1e-12)


def test_float32_mode_tracks_float64():
    hu = simple_phantom_hu(48, seed=5)
    vol = volume_from_hu(hu)
    proj = random_views(1, vol.center_in_world, seed=6, sphere_mm=0, sensor_size=(16, 16), pixel_size=3.0)[0]
    sc = oracle_scene([vol], proj, spectrum="120KV_AL43")
    r32 = sc.project("f32")
    r64 = sc.project("f64")
    e = rel_err(r32["intensity"], r64["intensity"])
    assert e.max() < 2e-3 and e.mean() < 2e-4
    assert r32["samples"] == pytest.approx(r64["samples"], rel=1e-3)


def test_priorities_select_the_winning_volume():
    """Nested cubes of one material: default priorities (last volume wins) give rho_B in the
    overlap; priorities [0, 1] let the outer cube win everywhere (project_kernel.cu:458-551)."""
    a = uniform_cube(32, 1.0)
    b = uniform_cube(16, 2.0)
    proj = axis_view((0, 1, 0), sensor=(4, 4), pixel=0.02)
    sc = oracle_scene([a, b], proj)
    v, u = _center_pixel(sc)
    ad = float(sc.project("f64")["area_density"][0, v, u]) * 10
    assert ad == pytest.approx(2.0 * 16 + 1.0 * 16, abs=0.5)
    sc = oracle_scene([a, b], proj, priorities=[0, 1])
    ad = float(sc.project("f64")["area_density"][0, v, u]) * 10
    assert ad == pytest.approx(1.0 * 32, abs=0.5)


def test_equal_priorities_reproduce_the_reference_accumulation_rule():
    """With equal priorities the reference's accumulation loop (project_kernel.cu:540-548) adds every
    traced volume of the winning priority, without re-checking its range: outside the inner cube the
    inner cube's clamped edge density is added with weight 1, inside both are averaged."""
    a = uniform_cube(32, 1.0)
    b = uniform_cube(16, 2.0)
    proj = axis_view((0, 1, 0), sensor=(4, 4), pixel=0.02)
    sc = oracle_scene([a, b], proj, priorities=[0, 0])
    v, u = _center_pixel(sc)
    for mode in ("f64", "f32"):
        ad = float(sc.project(mode)["area_density"][0, v, u]) * 10
        assert ad == pytest.approx((1.0 + 2.0) / 2 * 16 + (1.0 + 2.0) * 16, abs=0.6), mode


def test_attenuate_outside_adds_air_per_step():
    """attenuate_outside_volume: every step outside all volumes adds AIR_DENSITY (0.1129) to air,
    plus the source and detector tails (project_kernel.cu:358-361, 522-527, 557-560)."""
    vol = uniform_cube(16, 1.0, material="bone")
    proj = axis_view((0, 1, 0), sensor=(4, 4), pixel=0.05)
    sc0 = oracle_scene([vol], proj, attenuate=False)
    sc1 = oracle_scene([vol], proj, attenuate=True)
    r0 = sc0.project("f64")
    r1 = sc1.project("f64")
    # material list is [air, bone]; bone is unchanged
    np.testing.assert_allclose(r1["area_density"][1], r0["area_density"][0], rtol=1e-12)
    # air: (minAlpha + steps outside * step + (|r| - maxAlpha)) * 0.1129 / 10, and since the march
    # starts at minAlpha = |r| this is (|r| - chord) * 0.01129 within a step. With a unit-depth
    # world_from_index (|r| ~ 1 mm) the detector-side tail is negative, exactly as in the reference.
    v, u = _center_pixel(sc1)
    W = np.asarray(proj.world_from_index)[:3]
    r_len = np.linalg.norm(W @ np.array([u + 0.5, v + 0.5, 1.0]))
    expected = (r_len - 16.0) * 0.1129 / 10
    assert float(r1["area_density"][0, v, u]) == pytest.approx(expected, abs=2 * 0.1 * 0.01129)


def test_texture_emulation_quantises_filter_weights():
    """Linear filtering blends texels i = floor(x - 0.5) and i + 1 with weight frac(x - 0.5) held
    in 8 fractional bits; point filtering reads texel floor(x); both clamp."""
    vals = np.zeros((1, 1, 4), dtype=np.float32)
    vals[0, 0, :] = [0.0, 1.0, 0.0, 0.0]  # [nk][nj][ni], x = i
    dens = vals.transpose(2, 1, 0)  # [i, j, k]
    vol = [dict(density=dens, labels=np.zeros_like(dens, dtype=np.uint8), ijk_from_world=np.eye(4))]
    sc = oracle.Scene(vol, np.eye(3), np.zeros(3), width=1, height=1, step=0.1, energies=np.ones(1),
                      pdf=np.ones(1), mu=np.ones((1, 1)), frac_bits=8)
    for a in [0.0, 0.1, 0.25, 0.3337, 0.5, 0.999]:
        x = 0.5 + a  # blends texel 0 (0.0) and texel 1 (1.0) with weight a
        assert sc.tex_linear(0, x, 0.5, 0.5) == pytest.approx(np.floor(a * 256 + 0.5) / 256, abs=0)
    sc.sc.frac_bits = 0
    assert sc.tex_linear(0, 0.5 + 0.3337, 0.5, 0.5) == pytest.approx(0.3337, abs=1e-12)
    assert sc.tex_linear(0, -3.0, 0.5, 0.5) == 0.0  # clamp to texel 0
    assert sc.tex_linear(0, 1.5, 0.5, 0.5) == 1.0
    labs = np.zeros((4, 1, 1), dtype=np.uint8)
    labs[:, 0, 0] = [0, 1, 2, 3]
    vol = [dict(density=np.zeros((4, 1, 1), np.float32), labels=labs, ijk_from_world=np.eye(4))]
    sc = oracle.Scene(vol, np.eye(3), np.zeros(3), width=1, height=1, step=0.1, energies=np.ones(1),
                      pdf=np.ones(1), mu=np.ones((1, 4)))
    assert [sc.tex_point(0, x, 0, 0) for x in (-1.0, 0.0, 0.99, 1.0, 2.5, 3.999, 7.0)] == [0, 0, 0, 1, 2, 3, 3]


def test_ray_subset_matches_full_image():
    """Rays are independent: the oracle on a subset of pixel indices equals the full image there."""
    hu = simple_phantom_hu(40, seed=9)
    vol = volume_from_hu(hu)
    proj = random_views(1, vol.center_in_world, seed=2, sphere_mm=0, sensor_size=(10, 12), pixel_size=3.0)[0]
    sc = oracle_scene([vol], proj)
    full = sc.project("f32")
    ids = np.array([0, 5, 17, 63, 119], dtype=np.int64)
    sub = sc.project("f32", ray_ids=ids)
    np.testing.assert_array_equal(sub["intensity"], full["intensity"].ravel()[ids])
    np.testing.assert_array_equal(sub["area_density"], full["area_density"].reshape(3, -1)[:, ids])


def test_neglog_restatement():
    img = np.array([[[1.0, 2.0], [3.0, 4.0]]], dtype=np.float32)
    out = oracle.neglog(img)
    x = img + img.min() + 0.01
    y = -np.log(x)
    np.testing.assert_allclose(out, (y - y.min()) / (y.max() - y.min()), rtol=1e-6)
    const = oracle.neglog(np.ones((2, 3, 3), dtype=np.float32))
    assert np.all(const == 0)


def test_rays_that_miss_every_volume_are_unattenuated():
    """A ray that crosses no volume box samples nothing (project_kernel.cu:242-244, 321-334: maxAlpha
    stays 0, so num_steps <= 0): its photon_prob is sum(pdf) and its intensity sum(E pdf)."""
    vol = uniform_cube(8, 1.0, material="bone")
    proj = axis_view((0, 1, 0), sensor=(32, 4), pixel=2.0)  # ~1 mm per pixel at the cube: +-16 mm wide
    sc = oracle_scene([vol], proj, spectrum="90KV_AL40")
    e, pdf, _ = tables.build_tables("90KV_AL40", ["bone"], tables.NpzTables(GOLDEN_TABLES))
    e64, p64 = e.astype(np.float64), pdf.astype(np.float64)
    for mode, rtol in (("f64", 1e-12), ("f32", 1e-6)):
        r = sc.project(mode)
        for u in (0, 1, 30, 31):  # columns more than 4 mm off the axis
            assert np.all(r["area_density"][:, :, u] == 0), (mode, u)
            np.testing.assert_allclose(r["photon_prob"][:, u], p64.sum(), rtol=rtol)
            np.testing.assert_allclose(r["intensity"][:, u], (e64 * p64).sum(), rtol=rtol)
        assert np.all(r["area_density"][0, :, 15:17] > 0)  # the central columns cross the cube


def test_max_ray_length_ends_the_march():
    """max_ray_length caps every volume interval at alpha <= L (the slab test's upper bound,
    project_kernel.cu:265-323): with the source 500 mm from the centre of a 16 mm cube and L = 500 mm,
    the central ray crosses only the near half, 8 mm of it."""
    rho, step = 1.5, 0.1
    vol = uniform_cube(16, rho)
    proj = axis_view((0, 1, 0), sensor=(4, 4), pixel=0.02)
    full = oracle_scene([vol], proj, step=step)
    cut = oracle_scene([vol], proj, step=step, max_ray_length=500.0)
    v, u = _center_pixel(cut)
    for mode in ("f64", "f32"):
        ad_full = float(full.project(mode)["area_density"][0, v, u]) * 10
        ad_cut = float(cut.project(mode)["area_density"][0, v, u]) * 10
        assert ad_full == pytest.approx(rho * 16, abs=2 * step * rho), mode
        assert ad_cut == pytest.approx(rho * 8, abs=2 * step * rho), mode


def test_one_voxel_volume():
    """A 1 x 1 x 1 volume: the box is [-0.5, 0.5] in IJK and clamp addressing returns its one texel
    everywhere inside, so the central ray's path length is rho times the voxel's 3 mm."""
    rho, step = 2.0, 0.1
    vol = uniform_cube(1, rho, spacing=3.0)
    proj = axis_view((0, 1, 0), sensor=(4, 4), pixel=0.02)
    sc = oracle_scene([vol], proj, step=step)
    v, u = _center_pixel(sc)
    for mode in ("f64", "f32"):
        ad = float(sc.project(mode)["area_density"][0, v, u]) * 10
        assert ad == pytest.approx(rho * 3.0, abs=2 * step * rho), mode
