"""Build libmibm.so (CUDA C++ for sm_103a) in-tree.

Each translation unit under csrc/ is compiled by its own nvcc process (in
parallel) for ``-gencode arch=compute_103a,code=sm_103a`` and the objects are
linked into ``melt_ibm_gb300/_build/libmibm.so``.  Rebuilds only when a
source or header is newer than the library.

``build(bounds=True)`` makes the bounds build, ``_build/libmibm_bounds.so``
(``-DMIBM_BOUNDS``: kernels check their indices and count what they skip;
``mibm_bounds_check_`` reports it), a debug library beside the normal one.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmibm.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code (coordinate, wavenumber and line-solve tables) is compiled without
# floating-point contraction: gcc on Arm fuses a*b+c into FMAs by default,
# which moves knife-edge decisions of the reference's arithmetic (e.g. the
# MLS weight cut-off r > 1 when a marker sits exactly on a cell face).
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


# The Lagrangian kernels make discrete decisions (floor/nint of positions,
# signs of distances) from geometry; compiling them without FMA contraction
# keeps that arithmetic bit-identical to an IEEE evaluation in source order.
PER_FILE = {"lagr.cu": ["--fmad=false"], "interp.cu": ["--fmad=false"], "rigid.cu": ["--fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


LIB_BOUNDS = os.path.join(OUT, "libmibm_bounds.so")


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    deps = sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        [os.path.join(ROOT, "include", "mibm.h")]
    lib_t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > lib_t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None, bounds: bool = False) -> str:
    lib = LIB_BOUNDS if bounds else LIB
    if not force and not _stale(lib):
        return lib
    objdir = os.path.join(OUT, "bounds") if bounds else OUT
    os.makedirs(objdir, exist_ok=True)
    nvcc = _nvcc()
    extra = list(extra or []) + (["-DMIBM_BOUNDS"] if bounds else [])

    def compile_one(src: str) -> str:
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, *PER_FILE.get(os.path.basename(src), []), *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "--cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, bounds="--bounds" in sys.argv))
