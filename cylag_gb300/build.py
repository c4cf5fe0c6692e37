"""Build libcylag_gpu.so in-tree with nvcc for sm_103a (no torch extension
machinery, no cmake).  Translation units compile in parallel; the plain-form
kernels use -fmad=false so that FP64 arithmetic rounds exactly like the
reference's C.

A second library, ``libcylag_gpu_debug.so``, is the same code built with
-DCG_DEBUG_BOUNDS: every gather index read from the mesh tables or the
particle state is range-checked in the kernels (an out-of-range index sets
CG_ERR_BOUNDS and is redirected in bounds; nothing traps).  The Python layer
loads it instead of the normal library when CYLAG_DEBUG_BOUNDS=1.

Usage: ``python -m cylag_gb300.build [--force] [--debug-bounds]``
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_native"
LIB = OUT_DIR / "libcylag_gpu.so"
LIB_DEBUG = OUT_DIR / "libcylag_gpu_debug.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          f"-I{INCLUDE}", f"-I{CSRC}"]

# translation unit -> extra flags
# host code: no contraction either, so host-computed coefficients round as
# the reference's (e.g. 1/(rho_p + Ca rho_0), lagrangian_particle_set.pyx:371)
HOST_EXACT = ["-Xcompiler", "-ffp-contract=off"]
UNITS = {
    "cg_api.cu": ["-fmad=false", *HOST_EXACT],
    "cg_server.cu": HOST_EXACT,
    "cg_kernels_plain.cu": ["-fmad=false"],
    "cg_kernels_mixed.cu": [],
    "cg_lsm23_plain.cu": ["-fmad=false"],
    "cg_lsm23_mixed.cu": [],
    "cg_serve_plain.cu": ["-fmad=false"],
    "cg_serve_mixed.cu": [],
    "cg_sort.cu": [],
    "cg_snapshot.cpp": ["-Xcompiler", "-pthread"],
}
# cg_split3_form.cu: one object per form of the split 3D LSM3 and LSM2 steps
FORM_UNITS = [("cg_split3_form.cu", f"cg_split3_form_{k}", [f"-DCG_FORM={k}"]) for k in range(32)]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcylag_gpu.so")
    return exe


def _sources_newest() -> float:
    files = (list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) +
             list(CSRC.glob("*.cpp")))
    files += list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files)


def build(force: bool = False, verbose: bool = False, debug_bounds: bool = False) -> Path:
    lib = LIB_DEBUG if debug_bounds else LIB
    if not force and lib.exists() and lib.stat().st_mtime >= _sources_newest():
        return lib
    OUT_DIR.mkdir(exist_ok=True)
    objs = []
    exe = nvcc()
    flags = ["-DCG_DEBUG_BOUNDS"] if debug_bounds else []
    suffix = "_debug.o" if debug_bounds else ".o"

    def one(item):
        src, stem, extra = item
        obj = OUT_DIR / (stem + suffix)
        cmd = [exe, *ARCH, *COMMON, *flags, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout, r.stderr)
        return obj

    units = [(src, Path(src).stem, extra) for src, extra in UNITS.items()] + FORM_UNITS
    with ThreadPoolExecutor(max_workers=min(len(units), os.cpu_count() or 1)) as ex:
        objs = list(ex.map(one, units))
    tmp = lib.with_suffix(f".so.{os.getpid()}")
    cmd = [exe, *ARCH, "-shared", *map(str, objs), "-o", str(tmp), "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                debug_bounds="--debug-bounds" in sys.argv))
