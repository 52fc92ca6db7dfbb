"""bench.py's reference arm on the CPU: one JSON line with the keys the benchmark contract names.

The reference arm times the float64 port of the reference's stepping rule on the host cores; here it
runs on the small 128^3 / 256^2 workload for one warm-up and one timed step (a few seconds)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--small", "--steps", "1",
                          "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["unit"] == "projections/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"].startswith("simple128_det256")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_profile_figures_are_tied_to_the_forward_kernel_sources():
    """bench.py marks the ncu figures it reports as stale when the forward kernel's sources change:
    the files it hashes exist and are the ones the forward kernel's instantiation units include,
    and the committed figures carry a hash of that form."""
    sys.path.insert(0, str(ROOT))
    import bench

    csrc = ROOT / "deepdrr_gb300" / "csrc"
    for name in bench.FORWARD_SOURCES:
        assert (csrc / name).exists(), name
    # the instantiation units include the launch header, which includes the forward kernel's
    launch = (csrc / "drr_launch.cuh").read_text()
    assert '#include "drr_forward.cuh"' in launch
    forward = (csrc / "drr_forward.cuh").read_text()
    for inc in ("drr_alpha.h", "drr_coincide.h"):
        assert f'#include "{inc}"' in forward and inc in bench.FORWARD_SOURCES
    figures = bench.read_profile_figures()
    assert len(figures["source_sha"]) == len(bench.source_sha()) == 16
    assert 0 < figures["tex_pipe_pct"] <= 100 and figures["dram_bytes_per_launch"] > 0
