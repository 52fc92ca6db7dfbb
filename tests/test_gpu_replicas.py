"""The sharded adjoint: two ranks (gloo, one process each, both on cuda:0) each back-project their
own share of the views through autograd.project(..., distributed=True); the density and pose
gradients of the summed loss must equal the single-process gradient over all views.

The ranks' kernels never wait on one another: each rank runs its own forward and adjoint, and the
only exchange is a gloo all-reduce through host memory after its backward. Tolerance: 2e-5 of the
largest gradient entry (float32 atomic sums in a different order; one rank's partial sums are
added to the other's once more).
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch.distributed as dist
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

N_VIEWS = 6


def _gradients(rank=None, world=None):
    """Gradients of sum over views of ||I - target||^2 / N_VIEWS w.r.t. density and pose, over all
    views (rank None) or this rank's share (distributed)."""
    import deepdrr_gb300 as dd
    from deepdrr_gb300 import autograd, tables
    from deepdrr_gb300.phantoms import random_views, simple_phantom_hu, volume_from_hu
    from deepdrr_gb300.replicas import shard

    from helpers import GOLDEN_TABLES

    vol = volume_from_hu(simple_phantom_hu(40, seed=5))
    projs = random_views(N_VIEWS, vol.center_in_world, seed=6, sphere_mm=3.0, cone_deg=40.0, sensor_size=(48, 40),
                         pixel_size=2.0, fraction_range=(0.5, 0.6))
    views = projs if rank is None else shard(projs, rank, world)
    target_pose = np.array([1.5, -1.0, 0.5, 0.02, -0.03, 0.01])
    with dd.Projector([vol], spectrum="90KV_AL40", tables=tables.NpzTables(GOLDEN_TABLES), neglog=False,
                      step=0.1) as p:
        center = p.volume_center_world(0)
        ijk_t = np.asarray(vol.ijk_from_world.data) @ np.linalg.inv(autograd.rigid_motion(target_pose, center))
        target = p.project_tensors(*views, ijk_from_world=ijk_t[None, :3, :4])["intensity"].clone()
        d = torch.from_numpy(np.ascontiguousarray(vol.data, dtype=np.float32)).cuda().requires_grad_()
        pose = torch.zeros(6, dtype=torch.float64, requires_grad=True)
        out = autograd.project(p, *views, density=d, pose=pose, center=center, distributed=rank is not None)
        loss = ((out["intensity"] - target) ** 2).sum() / N_VIEWS
        loss.backward()
        torch.cuda.synchronize()
        return d.grad.cpu().numpy(), pose.grad.numpy(), [int(i) for i in range(len(views))]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        torch.cuda.set_device(0)
        gd, gp, mine = _gradients(rank, world)
        q.put((rank, gd, gp, len(mine)))
    except Exception as e:  # report instead of hanging the parent
        q.put((rank, None, repr(e), 0))
    finally:
        dist.destroy_process_group()


def test_two_ranks_sum_to_the_single_process_gradient():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted([q.get(timeout=300) for _ in range(world)], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, gd, gp, n in results:
        assert gd is not None, gp
    assert sum(n for _, _, _, n in results) == N_VIEWS
    want_d, want_p, _ = _gradients()
    scale_d = np.abs(want_d).max()
    scale_p = np.abs(want_p).max()
    assert scale_d > 0 and scale_p > 0
    for rank, gd, gp, _ in results:
        err_d = np.abs(gd - want_d).max() / scale_d
        err_p = np.abs(gp - want_p).max() / scale_p
        print(f"rank {rank}: density gradient within {err_d:.3g}, pose gradient within {err_p:.3g} of the "
              f"single-process gradient")
        assert err_d <= 2e-5 and err_p <= 2e-5
