"""Build recipe for the reference-kernel pin (TEST INFRASTRUCTURE ONLY).

1. ``build_cubins()`` compiles the reference's own ``deepdrr/projector/project_kernel.cu`` (with the
   ``-D`` macros deepdrr passes, projector.py:365-386) from the reference sources, where they lie,
   into ``oracle/_ref/projectKernel_nv{NV}_m{M}_att{A}[_mesh].cubin`` for sm_103a (``_mesh``:
   MESH_ADDITIVE_ENABLED=1, the build deepdrr makes when a projector has additive meshes). This
   needs the reference sources (``--reference``, default: the DEEPDRR_REFERENCE environment
   variable, else the checkout this recipe was written against) and runs only where they are
   present; the cubins are git-ignored and travel with the working tree.
2. ``build_harness()`` compiles ``oracle/ref_harness.cu`` (this project's driver for those cubins)
   into ``oracle/_build/libref_harness.so``. It needs only nvcc and libcuda.

    python oracle/build_ref.py [--reference PATH] [--harness-only]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
BUILD = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# (volumes, materials, ATTENUATE_OUTSIDE_VOLUME, MESH_ADDITIVE_ENABLED)
CONFIGS = ([(nv, m, att, 0) for nv in (1, 2, 3) for m in (2, 3, 4) for att in (0, 1)]
           + [(1, m, 0, 1) for m in (2, 3, 4)])
_FALLBACK_REFERENCE = "/root/reference"


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def cubin_path(n_volumes: int, n_materials: int, attenuate: bool, mesh_additive: bool = False) -> Path:
    tag = "_mesh" if mesh_additive else ""
    return REF_OUT / f"projectKernel_nv{n_volumes}_m{n_materials}_att{int(bool(attenuate))}{tag}.cubin"


def build_cubins(reference: Path) -> list[Path]:
    src = reference / "deepdrr" / "projector" / "project_kernel.cu"
    if not src.is_file():
        raise FileNotFoundError(f"reference kernel source not found: {src}")
    inc = [str(src.parent / "cubic"), str(src.parent)]
    REF_OUT.mkdir(parents=True, exist_ok=True)

    def one(cfg):
        nv, m, att, mesh = cfg
        out = cubin_path(nv, m, att, bool(mesh))
        if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
            return out
        defs = [f"-DNUM_VOLUMES={nv}", f"-DNUM_MATERIALS={m}", f"-DMESH_ADDITIVE_ENABLED={mesh}", "-DMAX_MESH_HITS=32",
                "-DMESH_LAYERS=2", f"-DATTENUATE_OUTSIDE_VOLUME={att}", "-DAIR_INDEX=0"]
        fd, tmp = tempfile.mkstemp(suffix=".cubin", dir=REF_OUT)
        os.close(fd)
        cmd = [_nvcc(), "-cubin", *ARCH, "-O3", *defs, "-I", inc[0], "-I", inc[1], str(src), "-o", tmp]
        subprocess.check_call(cmd)
        os.replace(tmp, out)
        return out

    with ThreadPoolExecutor(max_workers=8) as ex:
        return list(ex.map(one, CONFIGS))


def default_reference() -> Path:
    """Where the reference sources are read: $DEEPDRR_REFERENCE, else the recipe's own default."""
    return Path(os.environ.get("DEEPDRR_REFERENCE", _FALLBACK_REFERENCE))


def build_cubins_if_present() -> list[Path]:
    """Build the reference cubins when the reference sources exist here; otherwise keep whatever
    prebuilt cubins came with the tree."""
    ref = default_reference()
    if (ref / "deepdrr" / "projector" / "project_kernel.cu").is_file():
        return build_cubins(ref)
    return sorted(REF_OUT.glob("*.cubin"))


def harness_path() -> Path:
    return BUILD / "libref_harness.so"


def build_harness(force: bool = False) -> Path:
    src = HERE / "ref_harness.cu"
    out = harness_path()
    if out.exists() and not force and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    BUILD.mkdir(parents=True, exist_ok=True)
    fd, tmp = tempfile.mkstemp(suffix=".so", dir=BUILD)
    os.close(fd)
    cmd = [_nvcc(), *ARCH, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", str(src), "-o", tmp, "-lcuda"]
    subprocess.check_call(cmd)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(default_reference()))
    ap.add_argument("--harness-only", action="store_true")
    a = ap.parse_args()
    if not a.harness_only:
        for p in build_cubins(Path(a.reference)):
            print(p)
    print(build_harness())
