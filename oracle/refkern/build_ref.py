"""Compile the reference's own CUDA kernels into cubins under oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  The reference kernels are compiled from their
sources where they lie in the reference checkout (nothing is copied into this
repository), device code only, for sm_103a, with the reference's own nvcc
flags (setup.py: -O3 --use_fast_math).  The glm submodule that the sources
include is absent from the checkout, so the minimal column-major mat3 stand-in
under oracle/refkern/third_party/ takes its place.  The torch headers are
needed only because the sources include torch/extension.h next to their
kernels; nothing of torch ends up in device code.

The cubins carry no host code, so they load on either host architecture; the
tests and the benchmark load them through the CUDA driver API
(oracle/refkern/__init__.py).  Without the reference checkout this script does
nothing and the prebuilt cubins are used as they are.

    python oracle/refkern/build_ref.py [--force] [--src DIR]
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
# The reference checkout: GSTEX_REFERENCE if set, else a directory named
# "reference" beside this repository's root.
_REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE = os.environ.get("GSTEX_REFERENCE", os.path.join(os.path.dirname(_REPO), "reference"))
DEFAULT_SRC = os.path.join(REFERENCE, "gstex_cuda", "cuda", "csrc")

# cubin name -> reference source file (each holds the kernels named beside it)
UNITS = {
    "forward": "forward.cu",              # map_gaussian_to_intersects, get_tile_bin_edges
    "get_aabb_2d": "get_aabb_2d.cu",      # get_aabb_2d_kernel
    "texture": "texture.cu",              # texture_forward, texture_backward
    "texture_sample": "texture_sample.cu",  # texture_sample_forward, texture_sample_backward
    "texture_edit": "texture_edit.cu",    # texture_edit
    "sh": "bindings.cu",                  # compute_sh_forward_kernel, compute_sh_backward_kernel
}


def _torch_includes():
    import torch
    base = os.path.join(os.path.dirname(torch.__file__), "include")
    return [base, os.path.join(base, "torch", "csrc", "api", "include")]


def _compile(name: str, src: str, incs) -> str:
    out = os.path.join(OUT, name + ".cubin")
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--use_fast_math",
           "--expt-relaxed-constexpr", "-std=c++17", "-w", "-I" + HERE]
    cmd += ["-I" + d for d in incs]
    cmd += [src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
    return out


def build(force: bool = False, src_dir: str = DEFAULT_SRC) -> list:
    """Compile every unit whose cubin is missing (or all with force).  Returns
    the cubins written; an empty list when the reference checkout is absent."""
    if not os.path.isdir(src_dir):
        return []
    os.makedirs(OUT, exist_ok=True)
    todo = {n: os.path.join(src_dir, f) for n, f in UNITS.items()
            if force or not os.path.exists(os.path.join(OUT, n + ".cubin"))}
    if not todo:
        return []
    incs = _torch_includes() + [sysconfig.get_paths()["include"]]
    with ThreadPoolExecutor(max_workers=len(todo)) as ex:
        return list(ex.map(lambda kv: _compile(kv[0], kv[1], incs), todo.items()))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--src", default=DEFAULT_SRC)
    args = ap.parse_args()
    for p in build(args.force, args.src):
        print(p)
    sys.exit(0)
