"""Build the GB300 GQF native libraries in-tree with nvcc (sm_103a only).

Produces, under cqf_gb300/_lib/:
  libgqf_gb300.so         the C ABI of include/gqf.h (host API + kernels)
  libgqf_gb300_device.a   relocatable device code of the point API for
                          CUDA callers (include/gqf.cuh), link with -rdc=true

Translation units compile in parallel; no cmake.  Rebuilds only when a
source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
SO_PATH = os.path.join(LIB_DIR, "libgqf_gb300.so")
DEVLIB_PATH = os.path.join(LIB_DIR, "libgqf_gb300_device.a")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xptxas", "-O3", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cqf_gb300")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h*"))


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in _deps())


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile both libraries; return the shared-library path."""
    if not force and not _stale(SO_PATH) and not _stale(DEVLIB_PATH):
        return SO_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    nv = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = []
    for src in _sources():
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        jobs.append((src, obj, [nv, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]))
    dev_obj = os.path.join(OBJ_DIR, "gqf_point_rdc.o")
    jobs.append((None, dev_obj, [nv, *ARCH, *FLAGS, "-rdc=true", "-DGQF_DEVICE_LIBRARY_ONLY", "-c",
                                 os.path.join(CSRC, "gqf_point.cu"), "-o", dev_obj]))
    outs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(lambda j: _run(j[2]), jobs):
            outs.append(out)
    objs = [j[1] for j in jobs if j[0] is not None]
    tmp = SO_PATH + ".tmp"
    _run([nv, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, SO_PATH)
    tmpa = DEVLIB_PATH + ".tmp"
    _run([nv, *ARCH, "-lib", "-o", tmpa, dev_obj])
    os.replace(tmpa, DEVLIB_PATH)
    if verbose or ptxas_info:
        print("\n".join(o for o in outs if o.strip()))
    return SO_PATH


if __name__ == "__main__":
    import sys

    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(SO_PATH)
