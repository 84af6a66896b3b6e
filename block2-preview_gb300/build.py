"""Builds the CUDA library lib/libb2g.so for sm_103a (GB300) with nvcc.

Every translation unit in csrc/ is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into one
shared library exporting the C ABI of include/b2g.h.  Rebuilds only when a
source is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libb2g.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libb2g.so")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h")))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in sources() + headers() + [__file__])


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(LIBDIR, "obj", os.path.basename(src) + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "--cudart=static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


SHIM = os.path.join(HERE, "shim")
STAGED_BLOCK2 = os.path.join(SHIM, "_block2", "src")
SWEEP = os.path.join(LIBDIR, "dmrg_sweep")


def block2_source() -> str | None:
    """block2's headers for the drop-in: $BLOCK2_SRC (staged into
    shim/_block2/src so the tree can travel with this working copy), else an
    earlier staged copy, else None."""
    src = os.environ.get("BLOCK2_SRC")
    if src and os.path.isfile(os.path.join(src, "block2_core.hpp")):
        sys.path.insert(0, SHIM)
        import stage_block2

        if not os.path.isfile(os.path.join(STAGED_BLOCK2, "block2_core.hpp")):
            stage_block2.stage(src)
        return src
    if os.path.isfile(os.path.join(STAGED_BLOCK2, "block2_core.hpp")):
        return STAGED_BLOCK2
    return None


def _newer(target: str, deps) -> bool:
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def build_sweep_programs(verbose: bool = False, force: bool = False) -> dict:
    """Builds the DMRG sweep program twice, in parallel: lib/dmrg_sweep (block2
    with the GB300 drop-in, linked to libb2g.so) and oracle/_ref/dmrg_sweep_ref
    (block2's own CPU path, the reference arm).  Needs block2's headers
    (block2_source()); returns what was built or why not."""
    src = block2_source()
    if src is None:
        return {"skipped": "no block2 headers (set BLOCK2_SRC or stage them with shim/stage_block2.py)"}
    deps = [os.path.join(SHIM, f) for f in ("dmrg_sweep.cpp", "b2g_block2.hpp", "build.sh", "blas_defs.sh")]
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "dmrg_sweep_ref")
    jobs = []
    if force or _newer(SWEEP, deps + [LIB, os.path.join(ROOT, "include", "b2g.h")]):
        jobs.append((["bash", os.path.join(SHIM, "build.sh"), src, "gpu", SWEEP], SWEEP))
    if force or _newer(ref_bin, deps):
        jobs.append((["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), src], ref_bin))

    def run(job):
        cmd, out = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{' '.join(cmd)} failed:\n{r.stdout}\n{r.stderr}")
        return out

    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        done = list(ex.map(run, jobs))
    return {"built": done, "sweep": SWEEP, "reference": ref_bin}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    if "--sweep" in sys.argv:
        print(build_sweep_programs(verbose="-v" in sys.argv, force="--force" in sys.argv))
