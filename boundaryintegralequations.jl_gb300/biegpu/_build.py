"""Compile libbiegpu.so (CUDA, sm_103a) in-tree.

The library is built from the sources in ``csrc/`` with nvcc, one translation
unit per process in parallel, into ``biegpu/_lib/libbiegpu.so``.  Nothing is
installed into site-packages.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # boundaryintegralequations.jl_gb300/
CSRC = PKG_ROOT / "csrc"
LIB_DIR = Path(__file__).resolve().parent / "_lib"
OBJ_DIR = PKG_ROOT / "_build"
LIB_PATH = LIB_DIR / "libbiegpu.so"

SOURCES = [
    "bie_capi.cpp",
    "bie_setup.cpp",
    "bie_assemble.cu",
    "bie_assemble_mixed.cu",
    "bie_matvec.cu",
    "bie_solver.cu",
    "bie_nearfield.cpp",
    "bie_nearfield.cu",
    "bie_sweep.cu",
    "bie_adjoint.cu",
    "bie_lowp.cu",
    "bie_fastop.cu",
    "bie_peaks.cu",
    "bie_lossy.cpp",
    "bie_lossy.cu",
    "bie_mesh_io.cpp",
    "bie_multisolve.cu",
    "bie_cluster_gmres.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without FMA contraction so that the set-up arithmetic
# (quadrature rules, subdivision decisions, element geometry) rounds the same
# on x86-64 and aarch64 hosts; device code keeps nvcc's FMA contraction.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
          "-Xcompiler", "-fvisibility=hidden"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbiegpu.so")


def _sources_newer_than(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        [PKG_ROOT.parent / "include" / "biegpu.h"]
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and return the path of libbiegpu.so."""
    if not force and not _sources_newer_than(LIB_PATH):
        return LIB_PATH
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    # extra nvcc flags for tuning builds (e.g. "-DBIE_K2_MIN_BLOCKS=5")
    extra = os.environ.get("BIE_NVCC_EXTRA", "").split()

    def compile_one(src: str) -> Path:
        obj = OBJ_DIR / (src + ".o")
        cmd = [cc, *ARCH, *COMMON, *extra, "-I", str(PKG_ROOT.parent / "include"), "-c", str(CSRC / src),
               "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libbiegpu.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
