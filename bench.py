#!/usr/bin/env python
"""Benchmark of the DRR forward projector on one GB300 (or N independent replicas).

Headline workload (the production-size plain forward): a seeded 512 x 512 x 400 float32 CT
phantom at 0.8 x 0.8 x 1.0 mm (body, lungs, spine, ribs, titanium; materials air / bone / soft
tissue / titanium), a 1536 x 1536 detector at 0.194 mm, SDD 1020 mm, 32 seeded poses (point in a
100 mm ball, direction in a 30 degree cone, source-to-point fraction 0.5-0.9), 90 kVp spectrum
(151 bins), step 0.1 mm. One *step* renders the 32 views one launch per view.

  value     projections/s of the kernels with the volume resident in HBM (CUDA events on the
            launching stream, K timed steps after W warm-up steps, max over ranks)
  e2e       projections/s through the public API ``Projector.project(view)`` returning a host
            numpy image after GPU neglog (device->host copy of every image inside the timed region)
  roofline  the forward kernel against the measured HBM copy bandwidth: compulsory bytes per
            launch over its duration, with the ncu DRAM traffic of one launch beside it. The kernel
            is bound by instruction issue and the texture pipe, not HBM: ``tex_pipe`` carries the
            texture-pipe and issue utilisation of the latest ncu capture, marked stale when the
            kernel sources changed since

Baselines in the same line: ``reference_kernel`` times the reference's own projectKernel (compiled
from the reference sources, driven as _render_single drives it) on the same GPU and views;
``cpu_baseline`` times the oracle's float64 C restatement of its stepping rule on the host cores.

Unless ``--no-extra`` (or N > 1), the line also carries the other configurations, each measured in
this run with 3 warm-up and 3 timed steps:
  c1        128^3 phantom, one 256^2 view at 120 kVp (ours and the reference kernel)
  batched   3 volumes (512x512x400 CT, 256^3 phantom, 96x96x64 implant), 256 views at 384^2: one
            graph-captured persistent launch against plain launches, a per-view Projector.project
            loop, and the reference kernel
  adjoint   256^3 phantom, 64 views at 256^2: forward and forward + backward ms/view, memory
  half      512^3 CT, 32 views at 1536^2, 120 kVp, stored as float32 / float16 / bfloat16: speed,
            resident bytes, error against the float64 oracle

``--impl reference`` times the oracle's float64 C restatement of the reference stepping rule on
all host cores over a bounded ray sample (the reference projector itself only runs on a GPU,
through CuPy and an EGL context, which this machine does not have).
"""
from __future__ import annotations

import argparse
import hashlib
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
SUB_WARMUP, SUB_STEPS = 3, 3


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--views", type=int, default=None,
                    help="views per step (default: 32 for the headline; each configuration's own count alone)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--density-dtype", default="float32", choices=["float32", "float16", "bfloat16"])
    ap.add_argument("--workload", default="ct", choices=["ct", "ct512", "multi", "adjoint"],
                    help="ct: 512x512x400 CT, 90 kVp (default, with the other configurations as sub-objects); "
                         "ct512 / multi / adjoint: one configuration alone")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="headline only: no sub-objects, no reference kernel")
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
        return self

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


# ---------------------------------------------------------------- helpers -----------------------

def material_list(vols):
    return sorted({m for v in vols for m in v.materials[0]})


def remapped_labels(vol, mats):
    """Labels as indices into the sorted material list (projector.py:1495-1519)."""
    import numpy as np

    names, seg = vol.materials
    lut = np.zeros(max(names.values()) + 1, dtype=np.uint8)
    for n, i in names.items():
        lut[i] = mats.index(n)
    return lut[seg]


def scene_volumes(vols, mats):
    return [dict(density=v.data, labels=remapped_labels(v, mats), ijk_from_world=v.ijk_from_world.data) for v in vols]


FORWARD_SOURCES = ("drr_forward.cuh", "drr_launch.cuh", "drr_alpha.h", "drr_coincide.h", "drr_inst_nv1.cu",
                   "drr_inst_nv2.cu", "drr_inst_nv3.cu", "drr_inst_nv4.cu")


def source_sha() -> str:
    """Hash of the forward kernel's sources (the files its instantiation units compile from), to tell
    whether a saved ncu figure of that kernel still describes the current sources."""
    h = hashlib.sha256()
    for p in sorted(ROOT / "deepdrr_gb300" / "csrc" / name for name in FORWARD_SOURCES):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


def read_profile_figures() -> dict:
    out = {}
    if TRAFFIC_FILE.exists():
        for ln in TRAFFIC_FILE.read_text().splitlines():
            if ln.startswith("#") or ":" not in ln:
                continue
            key, _, val = ln.partition(":")
            key, val = key.strip(), val.strip()
            try:
                out[key] = val if key == "source_sha" else float(val)
            except ValueError:
                out[key] = val
    return out


def timed_events(fn, warmup: int, steps: int, stream) -> float:
    """Mean ms per call of fn, CUDA events on `stream`, after `warmup` untimed calls."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def reference_kernel_times(vols, projs, kw, *, views: int, repeats: int = 2) -> dict:
    """The reference's own projectKernel on `views` of these views: mean kernel ms per view (CUDA
    events, `repeats` launches per view after one untimed launch) and the host time of one whole
    _render_single sequence per view (geometry upload, launch, both read-backs, transposes)."""
    from deepdrr_gb300 import geo, tables
    from oracle import ref_kernel

    mats = material_list(vols)
    if not ref_kernel.available(len(vols), len(mats)):
        return {"unavailable": "reference cubins not built (no reference sources where this tree was built)"}
    e, pdf, mu = tables.build_tables(kw["spectrum"], mats, tables.NpzTables(TABLES))
    rs = ref_kernel.RefScene(scene_volumes(vols, mats), energies=e, pdf=pdf, mu=mu)
    ms, wall = [], []
    try:
        for pr in projs[:views]:
            W, s, w, h = geo.view_arrays(pr)
            r = rs.project(W, s, w, h, step=kw["step"], outputs=False, repeats=repeats, wall=True)
            ms.append(r["ms"])
            wall.append(r["wall_ms"])
    finally:
        rs.close()
    return {"views": len(ms), "ms_per_view": statistics.mean(ms), "projections_per_s": 1000.0 / statistics.mean(ms),
            "render_single_wall_ms_per_view": statistics.mean(wall),
            "source": "deepdrr/projector/project_kernel.cu:135-650 compiled for sm_103a with the reference's -D "
                      "macros, launched as projector.py:759-774 (8x8 blocks, one launch per view)"}


def cpu_baseline(vols, projs, kw, stride: int = 16, threads: int = 0):
    """Oracle float64 restatement of the reference stepping rule on a ray sample (every `stride`-th
    row and column of the first view), all host cores. Returns (projections/s, cores, sample)."""
    import numpy as np

    from deepdrr_gb300 import geo, tables
    from oracle import oracle

    src = tables.NpzTables(TABLES)
    mats = material_list(vols)
    e, pdf, mu = tables.build_tables(kw["spectrum"], mats, src)
    W, s, w, h = geo.view_arrays(projs[0])
    sc = oracle.Scene(scene_volumes(vols, mats), W, s, width=w, height=h, step=kw["step"], energies=e, pdf=pdf,
                      mu=mu, max_ray_length=-4.0)
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


def free_memory_bytes() -> int:
    """Free device memory, with torch's cache of freed blocks (the staging tensors of
    Projector.initialize) returned first, so that differences are what the library holds."""
    import torch

    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return int(torch.cuda.mem_get_info()[0])


# ---------------------------------------------------------------- --impl reference --------------

def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    vols, projs, kw, name = workload(args, 0)
    stride = 4 if not args.small else 1  # about 2.5 s of float64 work per step on 16 host cores
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


# ---------------------------------------------------------------- configurations ----------------

def phase_c1(args, local) -> dict:
    """128^3 phantom, one 256^2 view at 120 kVp: ours (plain launch) and the reference kernel."""
    import numpy as np
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import geo, metrics, phantoms, tables
    from oracle import ref_kernel

    vols, projs, kw = phantoms.workload_simple(seed=args.seed, views=1)
    p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=tables.NpzTables(TABLES), neglog=False,
                     cuda_device_id=local)
    p.initialize()
    stream = torch.cuda.current_stream()
    ms = timed_events(lambda: p.project_tensors(projs[0]), 20, 50, stream)
    ours = p.project_tensors(projs[0])["intensity"][0].cpu().numpy()
    samples = float(metrics.count_samples(vols, projs, kw["step"], -4.0, device=f"cuda:{local}").sum())
    p.free()
    out = {"workload": "simple128^3_det256_1view_120kV", "ms_per_view": ms, "projections_per_s": 1000.0 / ms,
           "gsamples_per_s": samples / (ms / 1000.0) / 1e9, "timing": "20 warm-up + 50 timed launches"}
    mats = material_list(vols)
    if ref_kernel.available(1, len(mats)):
        e, pdf, mu = tables.build_tables(kw["spectrum"], mats, tables.NpzTables(TABLES))
        rs = ref_kernel.RefScene(scene_volumes(vols, mats), energies=e, pdf=pdf, mu=mu)
        W, s, w, h = geo.view_arrays(projs[0])
        r = rs.project(W, s, w, h, step=kw["step"], repeats=50, wall=True)
        rs.close()
        rel = np.abs(ours.astype(np.float64) - r["intensity"]) / np.abs(r["intensity"].astype(np.float64))
        out["reference_kernel"] = {"ms_per_view": r["ms"], "projections_per_s": 1000.0 / r["ms"],
                                   "render_single_wall_ms_per_view": r["wall_ms"], "speedup": r["ms"] / ms,
                                   "max_rel_intensity_vs_ours": float(rel.max())}
    return out


def phase_batched(args, local, views: int = 256) -> dict:
    """Three volumes, 256 views at 384^2: graph-captured persistent launch vs plain launches, a
    per-view Projector.project loop and the reference kernel."""
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import metrics, phantoms, tables

    vols, projs, kw = phantoms.workload_multi(seed=args.seed, views=views)
    n = len(projs)
    W, H = projs[0].sensor_width, projs[0].sensor_height
    free0 = free_memory_bytes()
    p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=tables.NpzTables(TABLES), neglog=True,
                     cuda_device_id=local)
    p.initialize()
    resident = free0 - free_memory_bytes()
    stream = torch.cuda.current_stream()
    samples = float(metrics.count_samples(vols, projs, kw["step"], -4.0, device=f"cuda:{local}").sum())
    shape = p.autotune(*projs, max_views=64, cache=False)
    graph = p.capture(*projs, launch=shape)
    clocks = ClockSampler(local).start()
    ms_graph = timed_events(lambda: graph.launch(), SUB_WARMUP, SUB_STEPS, stream)
    clk = clocks.stop()
    ms_plain = timed_events(lambda: [p.project_tensors(pr) for pr in projs], SUB_WARMUP, SUB_STEPS, stream)
    graph.close()

    def wall(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(SUB_STEPS):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / SUB_STEPS

    e2e_batched = wall(lambda: p.project(*projs))
    e2e_loop = wall(lambda: [p.project(pr) for pr in projs])
    small = small_views_regime(p, vols, kw, local) if views >= 64 else None
    p.free()
    del graph, p
    torch.cuda.empty_cache()
    out = {"workload": f"multi3_ct512x512x400+256^3+96x96x64_det384_{n}views_90kV", "views_per_step": n,
           "graph_projections_per_s": n / (ms_graph / 1000.0), "plain_projections_per_s": n / (ms_plain / 1000.0),
           "speedup_graph_vs_plain": ms_plain / ms_graph, "gsamples_per_s": samples / (ms_graph / 1000.0) / 1e9,
           "autotuned_shape": shape, "resident_bytes": resident, "clocks": clk,
           "e2e": {"batched_projections_per_s": n / e2e_batched, "per_view_loop_projections_per_s": n / e2e_loop,
                   "speedup_batched_vs_per_view_loop": e2e_loop / e2e_batched,
                   "note": "Projector.project(*views) -> host numpy [256, 384, 384] after GPU neglog, against "
                           "[Projector.project(v) for v in views], the reference's serial pattern "
                           "(projector.py:679-685)", "d2h_bytes_per_step": n * W * H * 4},
           "timing": f"{SUB_WARMUP} warm-up + {SUB_STEPS} timed steps of {n} views"}
    ref = reference_kernel_times(vols, projs, kw, views=8)
    if "ms_per_view" in ref:
        ref["speedup_graph"] = ref["ms_per_view"] / (ms_graph / n)
        ref["speedup_plain"] = ref["ms_per_view"] / (ms_plain / n)
    out["reference_kernel"] = ref
    if small is not None:
        out["small_views"] = small
    return out


def small_views_regime(p, vols, kw, local, n: int = 2048, side: int = 32, seed: int = 17) -> dict:
    """The same three volumes seen by `n` views of side^2 pixels covering the 384^2 views' field:
    one view is too few rays to fill the GPU, so a plain launch per view is bound by the latency of
    its rays, and the persistent launch, which keeps every view's rays in flight together, is not."""
    import torch

    from deepdrr_gb300 import phantoms

    projs = phantoms.random_views(n, vols[0].center_in_world, seed=seed, sphere_mm=100.0, cone_deg=30.0,
                                  source_to_detector_distance=1020.0, pixel_size=0.3 * 384 / side,
                                  sensor_size=(side, side), fraction_range=(0.5, 0.9))
    stream = torch.cuda.current_stream()
    shape = p.autotune(*projs, max_views=256, cache=False)
    graph = p.capture(*projs, launch=shape)
    ms_graph = timed_events(lambda: graph.launch(), SUB_WARMUP, SUB_STEPS, stream)
    graph.close()
    ms_plain = timed_events(lambda: [p.project_tensors(pr) for pr in projs], 1, 1, stream)
    return {"workload": f"multi3_det{side}_{n}views_90kV", "views_per_step": n,
            "graph_projections_per_s": n / (ms_graph / 1000.0), "plain_projections_per_s": n / (ms_plain / 1000.0),
            "speedup_graph_vs_plain": ms_plain / ms_graph, "autotuned_shape": shape,
            "timing": f"graph: {SUB_WARMUP} warm-up + {SUB_STEPS} timed steps; plain: 1 + 1 steps of {n} launches"}



def phase_adjoint(args, local, views: int = 64) -> dict:
    """2D/3D registration step on the 256^3 phantom, 64 views at 256^2."""
    import numpy as np
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import autograd, tables
    from deepdrr_gb300.phantoms import workload_adjoint

    vols, projs, kw = workload_adjoint(seed=args.seed, views=views)
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
        for _ in range(SUB_WARMUP):
            fn()
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        ms = timed_events(fn, 0, SUB_STEPS, stream)
        return ms, torch.cuda.max_memory_allocated() - base

    clocks = ClockSampler(local).start()
    ms_fwd, _ = timed(lambda: step(False, backward=False))
    ms_stored, mem_stored = timed(lambda: step(False))
    ms_recompute, mem_recompute = timed(lambda: step(True))
    clk = clocks.stop()
    d = rho.detach().requires_grad_()
    pose = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    out = autograd.project(p, *projs, density=d, pose=pose, center=center)
    ((out["intensity"] - target) ** 2).mean().backward()
    g = pose.grad.numpy()
    cos = float(-(g @ kw["target_pose"]) / (np.linalg.norm(g) * np.linalg.norm(kw["target_pose"]) + 1e-30))
    M = len(p.all_materials)
    p.free()
    return {"workload": f"adjoint_phantom{vol.shape[0]}^3_det{W}_{n}views_90kV", "views_per_step": n,
            "loss": "MSE vs target at a pose perturbed <=5 mm / 5 deg", "gradients": "density (f32 volume) + 6-DoF pose",
            "fwd_ms_per_view": ms_fwd / n, "fwd_bwd_ms_per_view_stored": ms_stored / n,
            "fwd_bwd_ms_per_view_recompute": ms_recompute / n, "fwd_bwd_over_fwd": ms_stored / ms_fwd,
            "fwd_bwd_over_fwd_recompute": ms_recompute / ms_fwd,
            "memory_bytes": {"stored_peak": mem_stored, "recompute_peak": mem_recompute,
                             "area_density_held": n * M * W * H * 4},
            "pose_grad_cosine_to_target_direction": cos, "clocks": clk,
            "timing": f"{SUB_WARMUP} warm-up + {SUB_STEPS} timed steps of {n} views"}


def phase_half(args, local, views: int = 32) -> dict:
    """512^3 CT, 32 views at 1536^2, 120 kVp: float32 / float16 / bfloat16 density storage."""
    import numpy as np
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import metrics, phantoms, tables

    vols, projs, kw = phantoms.workload_ct(seed=args.seed, views=views, shape=(512, 512, 512), spectrum="120KV_AL43")
    stream = torch.cuda.current_stream()
    samples = float(metrics.count_samples(vols, projs, kw["step"], -4.0, device=f"cuda:{local}").sum())
    _, _, sample = cpu_baseline(vols, projs, kw, stride=8)
    ids, ref = cpu_baseline.last
    ids_t = torch.from_numpy(ids).to(f"cuda:{local}")
    out = {"workload": f"ct512x512x512_det1536_{len(projs)}views_120kV", "views_per_step": len(projs),
           "error_sample": sample.replace("extrapolated to whole views", "first view"),
           "timing": f"{SUB_WARMUP} warm-up + {SUB_STEPS} timed steps of 32 views per storage type"}
    for dt in ("float32", "float16", "bfloat16"):
        free0 = free_memory_bytes()
        p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=tables.NpzTables(TABLES), neglog=False,
                         density_dtype=dt, cuda_device_id=local)
        p.initialize()
        resident = free0 - free_memory_bytes()
        clocks = ClockSampler(local).start()
        ms = timed_events(lambda: [p.project_tensors(pr) for pr in projs], SUB_WARMUP, SUB_STEPS, stream)
        clk = clocks.stop()
        got = p.project_tensors(projs[0])["intensity"][0].flatten()[ids_t].double().cpu().numpy()
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-12)
        p.free()
        del p
        torch.cuda.empty_cache()
        out[dt] = {"projections_per_s": len(projs) / (ms / 1000.0), "ms_per_view": ms / len(projs),
                   "gsamples_per_s": samples / (ms / 1000.0) / 1e9, "resident_bytes": resident,
                   "max_rel_intensity_vs_float64": float(rel.max()), "mean_rel_intensity_vs_float64": float(rel.mean()),
                   "clocks": clk}
    return out


# ---------------------------------------------------------------- standalone configurations -----

def run_single(args, rank, world, local):
    import torch

    torch.cuda.set_device(local)
    fn = {"multi": phase_batched, "adjoint": phase_adjoint, "ct512": phase_half}[args.workload]
    res = fn(args, local) if args.views is None else fn(args, local, views=args.views)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "workload": args.workload, "n_gpus": world, **res}), flush=True)


# ---------------------------------------------------------------- the headline line -------------

def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if args.views is None:
            args.views = 32
        return run_reference(args, rank, world)
    if args.workload != "ct" and not args.small:
        return run_single(args, rank, world, local)

    import numpy as np
    import torch

    import deepdrr_gb300 as dd
    from deepdrr_gb300 import metrics, tables
    from deepdrr_gb300.replicas import max_over_ranks

    torch.cuda.set_device(local)
    if args.views is None:
        args.views = 32
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    extra = not args.no_extra and world == 1 and not args.small
    vols, projs, kw, name = workload(args, rank, world)
    src = tables.NpzTables(TABLES)
    nviews = len(projs)
    free0 = free_memory_bytes()
    p = dd.Projector(vols, spectrum=kw["spectrum"], step=kw["step"], tables=src, neglog=True,
                     density_dtype=args.density_dtype, cuda_device_id=local)
    p.initialize()
    resident = free0 - free_memory_bytes()
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
    clocks = ClockSampler(local).start()
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
    ms_b = timed_events(lambda: p.project_tensors(*projs), 2, args.steps, stream)

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
    hbm_peak = peaks.get("hbm_gbs")
    hbm_src = "of measured (MEASURED_PEAKS.json hbm_gbs)"
    if hbm_peak is None:
        hbm_peak, hbm_src = 6800.0, "of fallback (6.8 TB/s)"
    launch_s = ms_per_step / 1000.0 / nviews
    comp = metrics.compulsory_bytes(vols, W, H, args.density_dtype)
    prof = read_profile_figures()
    sha = source_sha()
    stale = prof.get("source_sha") != sha
    roofline = {"bound": "hbm", "achieved": comp / launch_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": comp / launch_s / 1e9 / hbm_peak, "traffic": prof.get("dram_bytes_per_launch"),
                "algorithmic_bytes_per_launch": comp,
                "note": "compulsory bytes (each voxel's density + label once, plus the output images) per view, peak "
                        f"{hbm_src}; traffic = ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                        f"(profiles/{TRAFFIC_FILE.name}). The kernel is issue- and texture-bound, see tex_pipe"}
    sampled_bytes = samples_per_step / nviews * metrics.BYTES_PER_SAMPLE[args.density_dtype]
    tex_pipe = {"tex_pipe_pct_of_peak_ncu": prof.get("tex_pipe_pct"), "issue_active_pct_ncu": prof.get("issue_active_pct"),
                "l1tex_hit_pct_ncu": prof.get("l1tex_hit_pct"), "l2_hit_pct_ncu": prof.get("l2_hit_pct"),
                "ncu_capture_of_this_build": not stale, "kernel_source_sha": sha,
                "sampled_bytes_per_launch": sampled_bytes, "sampled_gb_per_s": sampled_bytes / launch_s / 1e9,
                "note": "l1tex__data_pipe_tex_wavefronts and smsp__issue_active as % of peak in the ncu capture of one "
                        f"launch (profiles/{TRAFFIC_FILE.name}); sampled bytes = 40 B per sample at float32 "
                        "(8 density + 8 label texels), served by L1/TEX"}
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
        "ms_per_view": ms_per_step / nviews,
        "batched_projections_per_s": nviews / (ms_b / 1000.0),
        "resident_bytes": resident,
        "gpu_launches": nviews * args.steps,
        "clocks": clk,
        "roofline": roofline,
        "tex_pipe": tex_pipe,
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
    if extra:
        # ours on the same views the reference kernel is timed on, kernel time only
        n_ref = min(4, nviews)
        ms_ours = timed_events(lambda: [p.project_tensors(pr) for pr in projs[:n_ref]], 1, 2, stream) / n_ref
    p.free()
    del p
    torch.cuda.empty_cache()
    if extra:
        ref = reference_kernel_times(vols, projs, kw, views=n_ref)
        if "ms_per_view" in ref:
            ref["ours_ms_per_view_same_views"] = ms_ours
            ref["speedup"] = ref["ms_per_view"] / ms_ours
            if e2e is not None:
                ref["speedup_e2e"] = ref["render_single_wall_ms_per_view"] / (1000.0 / e2e["value"])
                ref["e2e_note"] = ("reference: geometry upload + kernel + read-back and transpose of intensity and "
                                   "photon_prob (its host neglog not counted); ours: Projector.project(view) with "
                                   "GPU neglog and the image read back")
        line["reference_kernel"] = ref
        del vols, projs
        line["c1"] = phase_c1(args, local)
        line["batched"] = phase_batched(args, local)
        line["adjoint"] = phase_adjoint(args, local)
        line["half"] = phase_half(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
