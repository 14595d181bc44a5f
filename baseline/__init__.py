"""The reference's own CUDA build, as a timed baseline -- BENCH/TEST
INFRASTRUCTURE, neither the product nor the oracle.

build() compiles the reference's device code (src/gqf.cu + src/hashutil.cu,
unmodified, from the reference tree) into baseline/_ref/gqf_ref_sm103a.cubin
and records the byte layout of its host structs (baseline/_ref/
refgpu_layout.json).  It needs the reference tree, so it runs where the tree
is; the outputs (git-ignored) travel with the repository to the GPU host,
where baseline/refgpu.py loads the cubin and drives its kernels.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference tree: $GQF_REFERENCE_TREE, else a checkout named "reference"
# beside this repository.
REFERENCE_TREE = os.environ.get("GQF_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                       "reference")
CCCL = "/usr/local/cuda/include/cccl"


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def build(ref: str = REFERENCE_TREE) -> str | None:
    """Builds the cubin and the layout file; returns the cubin path, or None
    where the reference tree is absent (the prebuilt files are then used)."""
    cubin = os.path.join(OUT, "gqf_ref_sm103a.cubin")
    layout = os.path.join(OUT, "refgpu_layout.json")
    if not os.path.isdir(ref):
        return cubin if os.path.exists(cubin) else None
    os.makedirs(OUT, exist_ok=True)
    nv = _nvcc()
    inc = ["-I" + os.path.join(ref, "src"), "-I" + os.path.join(ref, "include"), "-I" + CCCL]
    if not os.path.exists(cubin) or os.path.getmtime(cubin) < os.path.getmtime(os.path.join(HERE, "refgpu.cu")):
        subprocess.check_call([nv, "-std=c++17", "-O3", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                               *inc, "-w", os.path.join(HERE, "refgpu.cu"), "-o", cubin + ".tmp"])
        os.replace(cubin + ".tmp", cubin)
    if not os.path.exists(layout):
        with tempfile.TemporaryDirectory() as d:
            exe = os.path.join(d, "layout")
            subprocess.check_call([nv, "-std=c++17", *inc, "-w", os.path.join(HERE, "layout.cu"), "-o", exe])
            out = subprocess.check_output([exe], text=True)
        with open(layout + ".tmp", "w") as fh:
            fh.write(out)
        os.replace(layout + ".tmp", layout)
    return cubin
