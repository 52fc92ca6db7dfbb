"""GPU tests of the adjoint (density and 6-DoF pose gradients) and its autograd wrapper.

Tolerances (stated per test):
  * transposition <c, A rho> = <A^T c, rho> of the linear map density -> area densities: 1e-5
    relative to sum |c * A rho| (float32 forward and float32 atomics);
  * spectral chain: the adjoint fed dL/d(intensity), dL/d(photon_prob) equals the adjoint fed the
    float64 torch-autograd dL/d(area density) of the same Beer-Lambert sum, 1e-5 of max |grad|;
  * float64 autograd of the restatement in tests/fp64_reference.py, evaluated at the product's own
    float32 sample positions: density gradients per voxel within 1e-4 of the largest, pose
    gradients within 2e-3 of the largest component;
  * central finite differences (h = 1e-3): of that restatement for densities (1e-4), of the
    float64 oracle for the pose (see test_pose_gradient_... for the rotation tolerance).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import deepdrr_gb300 as dd
from deepdrr_gb300 import _lib, geo, tables
from deepdrr_gb300.autograd import project as project_ad, rigid_motion
from deepdrr_gb300.phantoms import random_views
from deepdrr_gb300.volume import Volume
from oracle import oracle

from fp64_reference import project_fp64_at_samples
from helpers import GOLDEN_TABLES, labels_for, material_list

pytestmark = pytest.mark.gpu

STEP = 0.1


def blob_volume(n=28, seed=0, margin=3):
    """Smooth density (sum of Gaussians) that is zero within `margin` voxels of the border, so
    that moving the volume slightly changes no entry or exit sample; bone where it is dense."""
    rng = np.random.default_rng(seed)
    g = np.indices((n, n, n)).astype(np.float64)
    d = np.zeros((n, n, n))
    for _ in range(5):
        c = rng.uniform(margin + 5, n - margin - 5, 3)
        s = rng.uniform(2.5, 5.0)
        d += rng.uniform(0.4, 1.2) * np.exp(-((g - c[:, None, None, None]) ** 2).sum(0) / (2 * s * s))
    d[:margin] = d[-margin:] = 0
    d[:, :margin] = d[:, -margin:] = 0
    d[:, :, :margin] = d[:, :, -margin:] = 0
    bone = d > 0.7
    vol = Volume.from_parameters(d.astype(np.float32), {"soft tissue": ~bone, "bone": bone},
                                 origin=-(n - 1) / 2 * np.ones(3), spacing=(1.0, 1.0, 1.0))
    return vol


def scene(views=3, seed=0, sensor=(24, 24)):
    vol = blob_volume(seed=seed)
    projs = random_views(views, vol.center_in_world, seed=seed + 11, sphere_mm=2.0, cone_deg=50.0,
                         sensor_size=sensor, pixel_size=2.5, fraction_range=(0.5, 0.55))
    return vol, projs


def projector(vol):
    return dd.Projector([vol], step=STEP, neglog=False, tables=tables.NpzTables(GOLDEN_TABLES))


def oracle_loss(vol, dens, ijk4, projs, a, b):
    """sum_views sum(a I + b P) from the float64 oracle."""
    src = tables.NpzTables(GOLDEN_TABLES)
    mats = material_list([vol])
    e, pdf, mu = tables.build_tables("90KV_AL40", mats, src)
    labels = labels_for(vol, mats)
    L = 0.0
    for k, proj in enumerate(projs):
        W, s, w, h = geo.view_arrays(proj)
        sc = oracle.Scene([dict(density=dens, labels=labels, ijk_from_world=ijk4)], W, s, width=w, height=h,
                          step=STEP, energies=e, pdf=pdf, mu=mu, max_ray_length=-1.0)
        r = sc.project("f64")
        L += float((a[k] * r["intensity"]).sum() + (b[k] * r["photon_prob"]).sum())
    return L


def test_adjoint_is_the_transpose_of_the_forward():
    vol, projs = scene()
    rng = np.random.default_rng(1)
    with projector(vol) as p:
        for trial in range(3):
            rho = torch.from_numpy(rng.uniform(0.0, 2.0, vol.shape).astype(np.float32)).cuda()
            p.set_density(rho)
            out = p.project_tensors(*projs, area_density=True)
            ad = out["area_density"]
            c = torch.from_numpy(rng.standard_normal(tuple(ad.shape)).astype(np.float32)).cuda()
            g = p.project_adjoint(*projs, area_density=ad, grad_area_density=c)["density"]
            lhs = float((c.double() * ad.double()).sum())
            rhs = float((g.double() * rho.double()).sum())
            scale = float((c.double() * ad.double()).abs().sum())
            print(f"transposition trial {trial}: lhs {lhs:.9g} rhs {rhs:.9g} rel {abs(lhs - rhs) / scale:.2e}")
            assert abs(lhs - rhs) <= 1e-5 * scale


def test_spectral_chain_matches_float64_autograd():
    vol, projs = scene()
    rng = np.random.default_rng(2)
    with projector(vol) as p:
        out = p.project_tensors(*projs, area_density=True)
        torch.cuda.synchronize()
        n, M, H, W = out["area_density"].shape
        a = torch.from_numpy(rng.standard_normal((n, H, W))).cuda()
        b = torch.from_numpy(rng.standard_normal((n, H, W))).cuda()
        E = torch.from_numpy(p._energies.astype(np.float64)).cuda()
        pdf = torch.from_numpy(p._pdf.astype(np.float64)).cuda()
        mu = torch.from_numpy(p._mu.astype(np.float64)).cuda()  # [bins][M]
        ad = out["area_density"].double().requires_grad_()
        x = torch.einsum("nmhw,bm->nbhw", ad, mu)
        e = torch.exp(-x) * pdf[None, :, None, None]
        I = (e * E[None, :, None, None]).sum(1)
        P = e.sum(1)
        assert torch.allclose(I.float(), out["intensity"], rtol=1e-5, atol=0)
        assert torch.allclose(P.float(), out["photon_prob"], rtol=1e-5, atol=0)
        ((a * I).sum() + (b * P).sum()).backward()
        g1 = p.project_adjoint(*projs, area_density=out["area_density"], grad_intensity=a.float().contiguous(),
                               grad_photon_prob=b.float().contiguous())["density"]
        g2 = p.project_adjoint(*projs, area_density=out["area_density"],
                               grad_area_density=ad.grad.float().contiguous())["density"]
        err = float((g1 - g2).abs().max() / g2.abs().max())
        print(f"spectral chain: max |g1 - g2| / max |g2| = {err:.2e}")
        assert err <= 1e-5


def scene_tables(vol):
    src = tables.NpzTables(GOLDEN_TABLES)
    mats = material_list([vol])
    e, pdf, mu = tables.build_tables("90KV_AL40", mats, src)
    return e, pdf, mu, labels_for(vol, mats)


def reference_loss(vol, projs, ijk_at, a, b, density, pose=None, center=None, filter="exact"):
    """sum_views sum(a I + b P) of the float64 autograd restatement at the product's own float32
    sample positions (taken with IJK_from_world = ijk_at, recorded by the float32 oracle)."""
    e, pdf, mu, labels = scene_tables(vol)
    L = 0.0
    for k, proj in enumerate(projs):
        W, s, w, h = geo.view_arrays(proj)
        sc = oracle.Scene([dict(density=vol.data, labels=labels, ijk_from_world=ijk_at)], W, s, width=w, height=h,
                          step=STEP, energies=e, pdf=pdf, mu=mu, max_ray_length=-1.0)
        samples = [sc.ray_samples(u, v) for v in range(h) for u in range(w)]
        I, P, _ = project_fp64_at_samples(density, labels, ijk_at, samples, w, h, STEP, e, pdf, mu, pose=pose,
                                          ijk0=np.asarray(vol.ijk_from_world.data), center=center, filter=filter)
        L = L + (torch.from_numpy(a[k]) * I).sum() + (torch.from_numpy(b[k]) * P).sum()
    return L


def test_density_gradient_matches_float64_autograd_and_finite_differences():
    vol, projs = scene()
    rng = np.random.default_rng(3)
    n = len(projs)
    H, W = projs[0].intrinsic.sensor_height, projs[0].intrinsic.sensor_width
    a = rng.standard_normal((n, H, W))
    b = rng.standard_normal((n, H, W))
    with projector(vol) as p:
        rho = torch.from_numpy(vol.data.astype(np.float32)).cuda().requires_grad_()
        out = project_ad(p, *projs, density=rho)
        L = (torch.from_numpy(a).cuda() * out["intensity"].double()).sum() + \
            (torch.from_numpy(b).cuda() * out["photon_prob"].double()).sum()
        L.backward()
        g = rho.grad.double().cpu()
    ijk0 = np.asarray(vol.ijk_from_world.data)
    d64 = torch.from_numpy(vol.data.astype(np.float64)).requires_grad_()
    reference_loss(vol, projs, ijk0, a, b, d64, filter="hw").backward()
    g_ref = d64.grad
    err = float((g - g_ref).abs().max() / g_ref.abs().max())
    print(f"density gradient vs float64 autograd: max |diff| / max |ref| = {err:.2e}")
    assert err <= 1e-4
    # central differences of the float64 restatement (linear in the densities along a direction)
    delta = torch.from_numpy(rng.standard_normal(vol.shape) * (vol.data > 0))
    h = 1e-3
    with torch.no_grad():
        base = torch.from_numpy(vol.data.astype(np.float64))
        lp = reference_loss(vol, projs, ijk0, a, b, base + h * delta, filter="hw")
        lm = reference_loss(vol, projs, ijk0, a, b, base - h * delta, filter="hw")
    fd = float((lp - lm) / (2 * h))
    an = float((g * delta).sum())
    print(f"density FD (h=1e-3) {fd:.9g} vs adjoint {an:.9g}: rel {abs(fd - an) / abs(fd):.2e}")
    assert abs(fd - an) <= 1e-4 * abs(fd)


@pytest.mark.parametrize("pose0", [np.zeros(6), np.array([0.4, -0.3, 0.2, 0.03, -0.02, 0.04])])
def test_pose_gradient_matches_float64_autograd_and_finite_differences(pose0):
    """Against the float64 autograd restatement at the product's own sample positions: 2e-3 of
    the largest component (the product's material weights come from the texture unit's 8-bit
    density filter, the restatement's from the exact one). Central differences (h = 1e-3) of the
    float64 oracle: translations within 5e-3 and rotations within 6e-2 of the largest component.
    The interpolant is trilinear, so its derivative jumps at voxel faces; a 1e-3 rad turn moves
    samples near the volume's rim by ~0.01 voxel and the central difference then mixes the slopes
    of neighbouring cells (it converges to the derivative as h shrinks)."""
    vol, projs = scene()
    rng = np.random.default_rng(4)
    n = len(projs)
    H, W = projs[0].intrinsic.sensor_height, projs[0].intrinsic.sensor_width
    a = rng.standard_normal((n, H, W))
    b = rng.standard_normal((n, H, W))
    with projector(vol) as p:
        center = p.volume_center_world(0)
        pose = torch.tensor(pose0, dtype=torch.float64, requires_grad=True)
        out = project_ad(p, *projs, pose=pose, center=center)
        L = (torch.from_numpy(a).cuda() * out["intensity"].double()).sum() + \
            (torch.from_numpy(b).cuda() * out["photon_prob"].double()).sum()
        L.backward()
        g = pose.grad.numpy()
    ijk0 = np.asarray(vol.ijk_from_world.data)
    ijk_at = ijk0 @ np.linalg.inv(rigid_motion(pose0, center))
    pr = torch.tensor(pose0, dtype=torch.float64, requires_grad=True)
    reference_loss(vol, projs, ijk_at, a, b, torch.from_numpy(vol.data.astype(np.float64)), pose=pr,
                   center=center).backward()
    g_ref = pr.grad.numpy()
    dens = vol.data.astype(np.float64)
    fd = np.zeros(6)
    h = 1e-3
    for k in range(6):
        e = np.zeros(6)
        e[k] = h
        lp = oracle_loss(vol, dens, ijk0 @ np.linalg.inv(rigid_motion(pose0 + e, center)), projs, a, b)
        lm = oracle_loss(vol, dens, ijk0 @ np.linalg.inv(rigid_motion(pose0 - e, center)), projs, a, b)
        fd[k] = (lp - lm) / (2 * h)
    print(f"pose gradient at {pose0}:\n  adjoint  {g}\n  autograd {g_ref}\n  fd       {fd}")
    scale = np.abs(g_ref).max()
    assert np.abs(g - g_ref).max() <= 2e-3 * scale
    assert np.abs(g[:3] - fd[:3]).max() <= 5e-3 * scale
    assert np.abs(g[3:] - fd[3:]).max() <= 6e-2 * scale


def test_recompute_matches_stored_area_densities():
    vol, projs = scene(views=2)
    with projector(vol) as p:
        rng = np.random.default_rng(5)
        out = p.project_tensors(*projs, area_density=True)
        gI = torch.from_numpy(rng.standard_normal(tuple(out["intensity"].shape)).astype(np.float32)).cuda()
        r1 = p.project_adjoint(*projs, area_density=out["area_density"], grad_intensity=gI, pose=True)
        r2 = p.project_adjoint(*projs, grad_intensity=gI, pose=True)
        for k in ("density", "pose"):
            err = float((r1[k] - r2[k]).abs().max() / r1[k].abs().max())
            assert err <= 1e-5, (k, err)
        # the autograd wrapper in recompute mode gives the same gradients
        rho = torch.from_numpy(vol.data.astype(np.float32)).cuda().requires_grad_()
        o = project_ad(p, *projs, density=rho, recompute=True)
        (o["intensity"] * gI).sum().backward()
        err = float((rho.grad - r1["density"]).abs().max() / r1["density"].abs().max())
        assert err <= 1e-5


def test_adjoint_rejects_unsupported_scenes():
    vol, projs = scene(views=1)
    vol2 = blob_volume(seed=1)
    with dd.Projector([vol, vol2], step=STEP, neglog=False, tables=tables.NpzTables(GOLDEN_TABLES)) as p:
        with pytest.raises(_lib.DrrError) as ei:
            p.project_adjoint(*projs)
        assert ei.value.status == _lib.DRR_ERR_UNSUPPORTED
    with dd.Projector([vol], step=STEP, neglog=False, tables=tables.NpzTables(GOLDEN_TABLES),
                      attenuate_outside_volume=True) as p:
        with pytest.raises(_lib.DrrError) as ei:
            p.project_adjoint(*projs)
        assert ei.value.status == _lib.DRR_ERR_UNSUPPORTED
