#!/usr/bin/env python
"""Benchmark of the DRR forward projector on one GB300 (or N independent replicas).

Workload (the production-size plain forward): a seeded 512 x 512 x 400 float32 CT phantom at
0.8 x 0.8 x 1.0 mm (body, lungs, spine, ribs, titanium; materials air / bone / soft tissue /
titanium), a 1536 x 1536 detector at 0.194 mm, SDD 1020 mm, 32 seeded poses (point in a 100 mm
ball, direction in a 30 degree cone, source-to-point fraction 0.5-0.9), 90 kVp spectrum
(151 bins), step 0.1 mm. One *step* renders the 32 views one launch per view.

  value  projections/s of the kernels with the volume resident in HBM (CUDA events on the
         launching stream, K timed steps after W warm-up steps, max over ranks)
  e2e    projections/s through the public API ``Projector.project(view)`` returning a host
         numpy image after GPU neglog (device->host copy of every image inside the timed region)

``--impl reference`` times the oracle's float64 C restatement of the reference stepping rule on
all host cores over a bounded ray sample (the reference projector itself only runs on a GPU
through CuPy + EGL, which this machine does not have).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DRR projections/s & Gsamples/s (512³ CT, 1536² det); fwd+adjoint ms/view"
TABLES = ROOT / "tests" / "golden" / "tables.npz"
PEAKS = ROOT / "MEASURED_PEAKS.json"
TRAFFIC_FILE = ROOT / "profiles" / "forward_ct512_det1536_dram.txt"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--views", type=int, default=32)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--density-dtype", default="float32", choices=["float32", "float16", "bfloat16"])
    ap.add_argument("--workload", default="ct", choices=["ct", "ct512", "multi", "adjoint"],
                    help="ct: 512x512x400 CT, 90 kVp (default); ct512: 512^3 CT, 120 kVp; "
                         "multi: 3 volumes, 256 views at 384^2, one graph-captured persistent launch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--small", action="store_true", help="a 128^3 / 256^2 workload for quick checks")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(args, rank: int, world: int = 1):
    """The seeded workload; under N ranks each renders its own contiguous share of N x views poses."""
    from deepdrr_gb300 import phantoms
    from deepdrr_gb300.replicas import shard

    if args.small:
        vols, projs, kw = phantoms.workload_simple(seed=args.seed, views=args.views)
        name = f"simple128_det256_{args.views}views_120kV"
    elif args.workload == "multi":
        vols, projs, kw = phantoms.workload_multi(seed=args.seed + rank, views=args.views)
        name = f"multi3_ct512x512x400+256^3+96x96x64_det384_{args.views}views_90kV"
    elif args.workload == "ct512":
        vols, projs, kw = phantoms.workload_ct(seed=args.seed, views=args.views * world, shape=(512, 512, 512),
                                               spectrum="120KV_AL43")
        projs = shard(projs, rank, world)
        name = f"ct512x512x512_det1536_{args.views}views_120kV"
    else:
        vols, projs, kw = phantoms.workload_ct(seed=args.seed, views=args.views * world)
        projs = shard(projs, rank, world)
        name = f"ct512x512x400_det1536_{args.views}views_90kV"
    return vols, projs, kw, name


def cpu_baseline(vols, projs, kw, stride: int = 16, threads: int = 0):
    """Oracle float64 restatement of the reference stepping rule on a ray sample (every `stride`-th
    row and column of the first view), all host cores. Returns (projections/s, cores, sample)."""
    import numpy as np

    from deepdrr_gb300 import geo, tables
    from oracle import oracle

    src = tables.NpzTables(TABLES)
    mats = sorted({m for v in vols for m in v.materials[0]})
    e, pdf, mu = tables.build_tables(kw["spectrum"], mats, src)
    W, s, w, h = geo.view_arrays(projs[0])
    vlist = []
    for v in vols:
        names, seg = v.materials
        lut = np.zeros(max(names.values()) + 1, dtype=np.uint8)
        for n, i in names.items():
            lut[i] = mats.index(n)
        vlist.append(dict(density=v.data, labels=lut[seg], ijk_from_world=v.ijk_from_world.data))
    sc = oracle.Scene(vlist, W, s, width=w, height=h, step=kw["step"], energies=e, pdf=pdf, mu=mu,
                      max_ray_length=-4.0)
    vv, uu = np.meshgrid(np.arange(0, h, stride), np.arange(0, w, stride), indexing="ij")
    ids = (vv * w + uu).ravel().astype(np.int64)
    cores = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = sc.project("f64", ray_ids=ids, threads=cores)
    dt = time.perf_counter() - t0
    frac = ids.shape[0] / float(w * h)
    cpu_baseline.last = (ids, ref["intensity"])  # the sample's float64 intensities, for error statements
    return frac / dt, cores, f"{ids.shape[0]} rays (every {stride}th row and column of one {w}x{h} view), " \
                             f"{dt:.2f} s, float64, extrapolated to whole views"


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    vols, projs, kw, name = workload(args, 0)
    stride = 2 if not args.small else 1  # about 10 s of float64 work per step on 16 host cores
    vals, dts = [], []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        pps, cores, sample = cpu_baseline(vols, [projs[k % len(projs)]], kw, stride=stride)
        if k >= args.warmup:
            vals.append(pps)
            dts.append(time.perf_counter() - t0)
    value = statistics.mean(vals)
    line = {
        "metric": METRIC, "value": value, "unit": "projections/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(dts),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded CT phantom, seeded poses)",
        "config": {"workload": name, "sample_stride": stride, "views_per_step": 1.0 / (stride * stride),
                   "step": "the rays of every stride-th row and column of one view, extrapolated to whole views"},
        "cpu_baseline": {"value": value, "unit": "projections/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "projections/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batched(args, rank, world, local):
    """Many views of several volumes: K graph replays of one persistent launch over all views
    (autotuned launch shape) against the same views rendered with one plain launch per view."""
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import metrics, tables

    torch.cuda.set_device(local)
    vols, projs, kw, name = workload(args, rank)
    p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=tables.NpzTables(TABLES), neglog=False,
                     density_dtype=args.density_dtype, cuda_device_id=local)
    p.initialize()
    stream = torch.cuda.current_stream()
    n = len(projs)
    W, H = projs[0].sensor_width, projs[0].sensor_height
    samples = float(metrics.count_samples(vols, projs, kw["step"], -4.0, device=f"cuda:{local}").sum())
    shape = p.autotune(*projs, max_views=min(n, 64), cache=False)
    graph = p.capture(*projs, launch=shape)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / args.steps

    clocks = ClockSampler(local)
    clocks.start()
    ms_graph = timed(lambda: graph.launch())
    clk = clocks.stop()
    ms_persistent = timed(lambda: p.project_tensors(*projs, persistent=True, launch=shape))
    ms_plain = timed(lambda: [p.project_tensors(pr) for pr in projs])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        p.project(*projs)
    torch.cuda.synchronize()
    e2e = n * args.steps / (time.perf_counter() - t0)
    graph.close()
    p.free()
    value = n / (ms_graph / 1000.0)
    line = {
        "metric": METRIC, "value": value, "unit": "projections/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantoms, seeded poses)",
        "config": {"workload": name, "views_per_step": n, "detector": [W, H], "launch": "persistent, CUDA graph",
                   "autotuned_shape": shape, "l2": "inputs larger than L2 (three volume textures, 0.9 GB)"},
        "gsamples_per_s": samples / (ms_graph / 1000.0) / 1e9,
        "persistent_projections_per_s": n / (ms_persistent / 1000.0),
        "plain_projections_per_s": n / (ms_plain / 1000.0),
        "speedup_vs_plain": ms_plain / ms_graph,
        "gpu_launches": 1, "clocks": clk,
        "e2e": {"value": e2e, "unit": "projections/s", "h2d_bytes_per_step": n * (9 + 3 + 12 * len(vols)) * 8,
                "d2h_bytes_per_step": n * W * H * 4},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_adjoint(args, rank, world, local):
    """2D/3D registration step: differentiable forward of all views, MSE against target images
    rendered at a perturbed pose, backward to the density volume and the 6-DoF pose. Timed with
    the area densities stored for the backward pass and with them recomputed there."""
    import numpy as np
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import autograd, tables
    from deepdrr_gb300.phantoms import workload_adjoint

    torch.cuda.set_device(local)
    vols, projs, kw = workload_adjoint(seed=args.seed + rank, views=args.views if args.views != 32 else 64)
    vol = vols[0]
    n = len(projs)
    W, H = projs[0].sensor_width, projs[0].sensor_height
    p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=tables.NpzTables(TABLES), neglog=False,
                     cuda_device_id=local)
    p.initialize()
    center = p.volume_center_world(0)
    ijk_t = np.asarray(vol.ijk_from_world.data) @ np.linalg.inv(autograd.rigid_motion(kw["target_pose"], center))
    target = p.project_tensors(*projs, ijk_from_world=ijk_t[None, :3, :4])["intensity"].clone()
    rho = torch.from_numpy(np.ascontiguousarray(vol.data, dtype=np.float32)).cuda()
    stream = torch.cuda.current_stream()

    def step(recompute, backward=True):
        d = rho.detach().requires_grad_()
        pose = torch.zeros(6, dtype=torch.float64, requires_grad=True)
        out = autograd.project(p, *projs, density=d, pose=pose, center=center, recompute=recompute)
        loss = ((out["intensity"] - target) ** 2).mean()
        if backward:
            loss.backward()
        return loss

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / args.steps, torch.cuda.max_memory_allocated() - base

    clocks = ClockSampler(local)
    clocks.start()
    ms_fwd, _ = timed(lambda: step(False, backward=False))
    ms_stored, mem_stored = timed(lambda: step(False))
    ms_recompute, mem_recompute = timed(lambda: step(True))
    clk = clocks.stop()
    # gradient sanity: one step's pose gradient points from the target pose back to zero
    d = rho.detach().requires_grad_()
    pose = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    out = autograd.project(p, *projs, density=d, pose=pose, center=center)
    ((out["intensity"] - target) ** 2).mean().backward()
    g = pose.grad.numpy()
    cos = float(-(g @ kw["target_pose"]) / (np.linalg.norm(g) * np.linalg.norm(kw["target_pose"]) + 1e-30))
    p.free()
    M = len(p.all_materials)
    line = {
        "metric": METRIC, "value": ms_stored / n, "unit": "ms/view (fwd+bwd)", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_stored, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantom, seeded poses)",
        "config": {"workload": f"adjoint_phantom{vol.shape[0]}^3_det{W}_{n}views_90kV", "views_per_step": n,
                   "detector": [W, H], "materials": M, "loss": "MSE vs target at a pose perturbed <=5 mm / 5 deg",
                   "gradients": "density (f32 volume) + 6-DoF pose",
                   "l2": "density texture 64 MB + 64 MB gradient volume; outputs re-read once"},
        "fwd_ms_per_view": ms_fwd / n,
        "fwd_bwd_ms_per_view_stored": ms_stored / n,
        "fwd_bwd_ms_per_view_recompute": ms_recompute / n,
        "bwd_over_fwd": (ms_stored - ms_fwd) / ms_fwd,
        "fwd_bwd_over_fwd": ms_stored / ms_fwd,
        "memory_bytes": {"stored_peak": mem_stored, "recompute_peak": mem_recompute,
                         "area_density_held": n * M * W * H * 4},
        "pose_grad_cosine_to_target_direction": cos,
        "gpu_launches": 2 * n // 32 + 2, "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "multi":
        return run_batched(args, rank, world, local)
    if args.workload == "adjoint":
        return run_adjoint(args, rank, world, local)

    import numpy as np
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import metrics, tables
    from deepdrr_gb300.replicas import max_over_ranks

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    vols, projs, kw, name = workload(args, rank, world)
    src = tables.NpzTables(TABLES)
    nviews = len(projs)
    p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=src, neglog=True,
                     density_dtype=args.density_dtype, cuda_device_id=local)
    p.initialize()
    W, H = projs[0].sensor_width, projs[0].sensor_height
    samples = metrics.count_samples(vols, projs, kw["step"], -4.0, device=f"cuda:{local}")
    samples_per_step = float(samples.sum())
    stream = torch.cuda.current_stream()

    def step_plain():
        for pr in projs:
            p.project_tensors(pr)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step_plain()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_plain()
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), device="cuda")
    ms_per_step = ms / args.steps
    value = nviews * world * args.steps / (ms / 1000.0)
    gsamples = samples_per_step * world * args.steps / (ms / 1000.0) / 1e9

    # batched: all views of a step in one library call
    for _ in range(2):
        p.project_tensors(*projs)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        p.project_tensors(*projs)
    e1.record(stream)
    e1.synchronize()
    ms_b = e0.elapsed_time(e1) / args.steps

    # end to end through the public API (host numpy out, neglog on the GPU)
    e2e = None
    if not args.no_e2e:
        for pr in projs[:2]:
            p.project(pr)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for pr in projs:
                img = p.project(pr)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        geometry_bytes = nviews * (9 + 3 + 12 * len(vols)) * 8
        e2e = {"value": nviews * args.steps * world / dt, "unit": "projections/s",
               "h2d_bytes_per_step": geometry_bytes, "d2h_bytes_per_step": nviews * W * H * 4}

    # roofline of the forward kernel: compulsory HBM bytes per launch (one view) over its duration
    peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    comp = metrics.compulsory_bytes(vols, W, H, args.density_dtype)
    launch_s = ms_per_step / 1000.0 / nviews
    achieved = comp / launch_s / 1e9
    traffic = tex_pipe = l1_hit = l2_hit = None
    if TRAFFIC_FILE.exists():
        for ln in TRAFFIC_FILE.read_text().splitlines():
            key, _, val = ln.partition(":")
            if key == "dram_bytes_per_launch":
                traffic = float(val)
            elif key == "tex_pipe_pct":
                tex_pipe = float(val)
            elif key == "l1tex_hit_pct":
                l1_hit = float(val)
            elif key == "l2_hit_pct":
                l2_hit = float(val)
    sampled_bytes = samples_per_step / nviews * metrics.BYTES_PER_SAMPLE[args.density_dtype]
    line = {
        "metric": METRIC, "value": value, "unit": "projections/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"float32": "f32", "float16": "f16-storage/f32",
                                       "bfloat16": "bf16-storage/f32"}[args.density_dtype],
        "data": "synthetic (seeded CT phantom with titanium; seeded C-arm poses)",
        "config": {"workload": name, "volume": list(vols[0].shape), "detector": [W, H], "views_per_step": nviews,
                   "materials": len(p.all_materials), "n_bins": int(p._energies.shape[0]), "step_mm": kw["step"],
                   "density_dtype": args.density_dtype, "launch": "plain: one launch per view",
                   "parallelism": f"replicas x{world} (views sharded, no collective)",
                   "l2": "inputs larger than L2 (volume textures > 129 MB)"},
        "gsamples_per_s": gsamples,
        "samples_per_view": samples_per_step / nviews,
        "batched_projections_per_s": nviews / (ms_b / 1000.0),
        "gpu_launches": nviews * args.steps,
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "algorithmic_bytes_per_launch": comp,
                     "note": "compulsory bytes (each voxel's density+label once, plus output images) per view; "
                             "peak = measured copy bandwidth of MEASURED_PEAKS.json"},
        "sampled": {"bytes_per_launch": sampled_bytes, "gb_per_s": sampled_bytes / launch_s / 1e9,
                    "tex_pipe_pct_of_peak_ncu": tex_pipe, "l1tex_hit_pct_ncu": l1_hit, "l2_hit_pct_ncu": l2_hit,
                    "note": "texel bytes the march reads per view (40 B/sample at float32), served by L1/TEX; "
                            "texture-pipe utilisation from the ncu capture in profiles/"},
        "e2e": e2e,
    }
    if rank == 0 and not args.no_cpu_baseline:
        pps, cores, sample = cpu_baseline(vols, projs, kw, stride=2 if not args.small else 1)
        line["cpu_baseline"] = {"value": pps, "unit": "projections/s", "cores": cores, "kind": "port",
                                "sample": sample}
        # error of this run's first view against the float64 oracle on the same rays
        ids, ref = cpu_baseline.last
        got = p.project_tensors(projs[0])["intensity"][0].flatten()[torch.from_numpy(ids).to(f"cuda:{local}")]
        rel = np.abs(got.double().cpu().numpy() - ref) / np.maximum(np.abs(ref), 1e-12)
        line["error_vs_float64"] = {"max_rel_intensity": float(rel.max()), "mean_rel_intensity": float(rel.mean()),
                                    "rays": int(ids.shape[0])}
    p.free()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
