"""Builds libhairfb.so (the CUDA kernels + C-ABI) in-tree with nvcc.

    python -m hairfb.build           # from frostbitten-hair-webgpu_gb300/

Each translation unit is compiled for sm_103a only, in parallel, then linked
into ``hairfb/_lib/libhairfb.so``.  The library is compiled with
``-fmad=false -prec-div=true -prec-sqrt=true``: every kernel evaluates its
fp32 expressions one IEEE operation at a time, which is what makes the
integer outputs of the passes (tile lists, depth bounds, grids) reproducible.
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
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libhairfb.so")
OBJ_DIR = os.path.join(ROOT, "_build")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]
SOURCES = ["hfb_api.cu", "sim.cu", "shading.cu", "raster.cu", "noalloc.cu", "batch.cu", "hairdepth.cu", "present.cu", "ao.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhairfb.so")


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(ROOT), "include", "hairfb.h"))
    return hs


CHECKED_LIB = os.path.join(OUT_DIR, "libhairfb_checked.so")


def build(force: bool = False, verbose: bool = False, extra_flags=(), checked: bool = False) -> str:
    """Builds libhairfb.so; with ``checked``, the self-checking variant
    libhairfb_checked.so (device index checks that print and skip, for
    diagnosing a fault; select it with HAIRFB_LIBRARY)."""
    obj_dir, lib = (os.path.join(ROOT, "_build", "checked"), CHECKED_LIB) if checked else (OBJ_DIR, LIB)
    if checked:
        extra_flags = tuple(extra_flags) + ("-DHFB_DEVICE_CHECKS",)
    return _build(force, verbose, extra_flags, obj_dir, lib)


def _build(force, verbose, extra_flags, OBJ_DIR, LIB) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    hdrs = _headers()
    cc = nvcc()

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        if force or _stale(o, [s, *hdrs]):
            cmd = [cc, *GENCODE, *NVCC_FLAGS, *extra_flags, "-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [cc, *GENCODE, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
