"""Build recipe for the unmodified reference CyLag (Cython) as a test oracle.

Test infrastructure only: nothing in the product imports what this builds.

Two stages, so that the compiled reference can exist on machines that have
neither Cython nor the reference sources:

1. ``generate`` (needs Cython and the reference tree): cythonize every
   ``cylag/**/*.pyx`` of the reference, read in place, with the compiler
   directives of the reference's standard build (boundscheck, wraparound,
   cdivision, language_level 3; reference ``setup.py:59-71``), writing the
   generated C into ``oracle/_ref/gen/`` and the pure-Python package files
   (``__init__.py``, ``cylag_dico.py``) into ``oracle/_ref/cylag/``.
2. ``compile`` (needs only gcc and the Python headers): compile each generated
   C file with ``-O2 -fno-fast-math -ffp-contract=off`` (x86-64 gcc does not
   contract to FMA at -O2; on aarch64 contraction is on by default and would
   change the reference's rounding) into an extension module under
   ``oracle/_ref/cylag/``.

Importing the result needs ``oracle/_ref`` and ``oracle/ref_stubs`` on
``sys.path`` (see ``oracle/refpath.py``).

Usage: ``python oracle/build_ref.py [--src DIR] [--jobs N]`` (DIR defaults to
``$CYLAG_REFERENCE_SRC``, else the reference tree's mount point here).
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
GEN = OUT / "gen"
PKG = OUT / "cylag"

DIRECTIVES = {
    "boundscheck": True,
    "wraparound": True,
    "initializedcheck": False,
    "nonecheck": False,
    "cdivision": True,
    "language_level": 3,
}


def generate(src: Path) -> None:
    """Cythonize the reference package read in place under ``src``."""
    from Cython.Build import cythonize  # only needed for this stage

    pyx = sorted((src / "cylag").rglob("*.pyx"))
    if not pyx:
        raise FileNotFoundError(f"no .pyx under {src}/cylag")
    GEN.mkdir(parents=True, exist_ok=True)
    cwd = os.getcwd()
    os.chdir(src)  # cythonize resolves package-relative cimports from here
    try:
        rel = [str(p.relative_to(src)) for p in pyx]
        cythonize(rel, compiler_directives=DIRECTIVES, build_dir=str(GEN),
                  nthreads=os.cpu_count() or 1, quiet=True)
    finally:
        os.chdir(cwd)
    for py in (src / "cylag").rglob("*.py"):
        dst = PKG / py.relative_to(src / "cylag")
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(py, dst)


def _compile_one(c_file: Path) -> str:
    rel = c_file.relative_to(GEN / "cylag").with_suffix("")
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    out = PKG / (str(rel) + suffix)
    if out.exists() and out.stat().st_mtime >= c_file.stat().st_mtime:
        return f"up-to-date {rel}"
    out.parent.mkdir(parents=True, exist_ok=True)
    inc = sysconfig.get_paths()["include"]
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fno-fast-math",
           "-ffp-contract=off", "-fno-strict-aliasing", "-w",
           f"-I{inc}", str(c_file), "-o", str(out)]
    subprocess.run(cmd, check=True)
    return f"built {rel}"


def compile_all(jobs: int) -> None:
    cfiles = sorted((GEN / "cylag").rglob("*.c"))
    if not cfiles:
        raise FileNotFoundError(f"no generated C under {GEN}; run generate first")
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for msg in ex.map(_compile_one, cfiles):
            pass


def default_src() -> Path:
    """The reference tree: $CYLAG_REFERENCE_SRC, else where this machine
    mounts it."""
    return Path(os.environ.get("CYLAG_REFERENCE_SRC", "/root/reference"))


def sources_present() -> bool:
    return (default_src() / "cylag").is_dir()


def generated_present() -> bool:
    """The generated C (stage 1's output) is here: stage 2 can run."""
    return any((GEN / "cylag").rglob("*.c")) if (GEN / "cylag").is_dir() else False


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=str(default_src()))
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--stage", choices=["all", "generate", "compile"], default="all")
    a = ap.parse_args(argv)
    src = Path(a.src)
    if a.stage in ("all", "generate"):
        if not (src / "cylag").is_dir():
            print(f"reference sources not found at {src}; skipping generate")
        else:
            generate(src)
    if a.stage in ("all", "compile"):
        compile_all(a.jobs)
    return 0


if __name__ == "__main__":
    sys.exit(main())
