"""Builds libmsplat_gb300.so in-tree with nvcc for sm_103a (GB300).

Translation units compile in parallel.  The files whose float results decide
integer outputs or must match the oracle bit for bit (projection, tile
mapping, forward raster) are built with --fmad=false: there every product is
rounded before it is added, and fused only where the source says fmaf.  Host
code is built with -ffp-contract=off so that its float results (camera
matrices, metrics, seed scales) are the same on x86-64 and AArch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmsplat_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NO_FMAD = {"project_fwd.cu", "tiles.cu", "raster_fwd.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _flags(src: str):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                "-Xcompiler", "-ffp-contract=off",
                "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    if src in NO_FMAD:
        f.append("--fmad=false")
    if os.environ.get("MSPLAT_CHECKED"):
        f.append("-DMSPLAT_CHECKED")
    return f


def _flavor() -> str:
    return "checked" if os.environ.get("MSPLAT_CHECKED") else "release"


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, _flavor(), src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "msplat_engine.h"))
    deps.append(os.path.join(ROOT, "include", "msplat_c_api.h"))
    deps.append(os.path.abspath(__file__))   # flags live here
    if os.path.exists(obj) and all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in deps if os.path.exists(d)):
        return obj
    cmd = [nvcc()] + _flags(src) + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(os.path.join(BUILD, _flavor()), exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    stamp = os.path.join(BUILD, "linked_flavor")
    last = open(stamp).read() if os.path.exists(stamp) else ""
    if (not os.path.exists(LIB) or last != _flavor()
            or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        with open(stamp, "w") as f:
            f.write(_flavor())
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
