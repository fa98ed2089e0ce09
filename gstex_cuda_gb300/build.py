"""Compile the CUDA library for sm_103a into gstex_cuda_gb300/_build/.

Each translation unit is compiled by nvcc in parallel and the objects are
linked into libgstex_gb300.so (static CUDA runtime, C ABI declared in
include/gstex_gb300.h).  Rebuilds only when a source or header is newer than
the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgstex_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", os.path.join(REPO, "include")]
# Per-file arithmetic flags: projection/binning must be reproducible bit for
# bit (no contraction, IEEE division); the compositor uses fast math like the
# reference build (setup.py:64-76 of the reference project).
PER_FILE = {
    "project.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    "binning.cu": ["-fmad=false", "-prec-div=true"],
    "raster.cu": ["--use_fast_math"],
    "batch.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    "sample.cu": ["-fmad=false"],
    "status.cu": [],
    "sort_static.cu": [],
    "preprocess.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the gstex_gb300 CUDA library cannot be built")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(REPO, "include", "*.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    flags = PER_FILE.get(os.path.basename(src), []) + os.environ.get("GSTEX_NVCC_EXTRA", "").split()
    cmd = [nvcc()] + ARCH + COMMON + flags + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Build the library if needed and return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
