"""Builds the in-tree CUDA library ``wem-fwi_gb300/wemgpu/_lib/libwemgpu.so``.

One nvcc invocation per translation unit (compiled in parallel), one
``-gencode`` for sm_103a, no cmake.  The library is the only compute path of
the package: nothing falls back to the CPU when it is missing.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libwemgpu.so")
OBJ_DIR = os.path.join(OUT_DIR, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["kernels.cu", "kernels_w.cu", "tables.cu", "timefreq.cu", "grad.cu", "offset.cu", "k3d.cu", "noalloc.cu",
           "interp.cu", "rowops.cu", "api.cpp", "planner.cpp", "cmap.cpp"] + [
    f"kw_e{e}_{p}.cu" for e in (32, 24, 16, 12, 8) for p in ("adj", "adj1", "wem", "fwd", "grad", "off")] + [
    f"k3_e{e}.cu" for e in (32, 24, 16, 12, 8)]

# host code whose float results must not depend on the machine: the
# conformal maps turn float coordinates into grid indices, so no multiply-add
# may be fused on one machine and not on another
HOST_EXACT = {"cmap.cpp"}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build wemgpu")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "wemgpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    os.makedirs(OBJ_DIR, exist_ok=True)
    # stream 0 of every launch and runtime call is the calling thread's
    # default stream: host threads that drive separate engines run on the
    # GPU concurrently (the per-thread default stream still synchronises with
    # the legacy default stream other libraries use)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "--default-stream", "per-thread",
              "-DCUDA_API_PER_THREAD_DEFAULT_STREAM=1", "-I", INCLUDE, "-I", CSRC]

    def compile_one(src: str) -> str:
        obj = os.path.join(OBJ_DIR, src + ".o")
        cmd = [nvcc, *common, "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd[1:1] = [*ARCH, "-lineinfo", "-Xptxas", "-v"] if verbose else [*ARCH, "-lineinfo"]
        if src in HOST_EXACT:
            cmd[1:1] = ["-Xcompiler", "-ffp-contract=off"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
