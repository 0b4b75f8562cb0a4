"""Build libpm_gb300.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process, in parallel; the spectral
kernels are compiled once per supported grid size.  Objects go to ``_build/`` at the
repository root and the shared library next to this file.  A rebuild happens only
when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(REPO, "_build")
LIB = os.path.join(PKG, "libpm_gb300.so")

GRID_SIZES = (16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ("pm_api.cu", "pm_batch.cu", "pm_particles.cu", "pm_sort.cu", "pm_spectral_host.cu", "pm_noalloc.cu",
           "pm_ics.cu", "pm_diagnostics.cu")


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", ARCH, "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE]


def _units():
    units = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        if os.path.exists(src):
            units.append((src, os.path.join(BUILD, s.replace(".cu", ".o")), []))
    for n in GRID_SIZES:
        units.append((os.path.join(CSRC, "pm_spectral_n.cu"), os.path.join(BUILD, f"pm_spectral_{n}.o"),
                      [f"-DPM_N={n}"]))
    return units


def _newest_input():
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return max(t, os.path.getmtime(__file__))


def up_to_date():
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link the engine; returns the path of the shared library."""
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    units = _units()
    jobs = jobs or max(1, min(len(units), os.cpu_count() or 4))

    def compile_one(u):
        src, obj, extra = u
        cmd = [nvcc, *_flags(), *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(obj)}:\n{r.stderr[-4000:]}")
        if verbose:
            print("built", os.path.basename(obj), file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
