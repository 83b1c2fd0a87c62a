"""Builds libatmo_gb300.so (the CUDA kernels for sm_103a and the C ABI of
include/atmo/atmo.h) in-tree with nvcc, compiling the translation units in
parallel."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libatmo_gb300.so")
# The checked build (device-side index checks, csrc/atmo_check.cuh): the same
# sources compiled with -DATMO_DEVICE_CHECKS into their own objects.
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "libatmo_gb300_checked.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "-Xptxas", "-warn-spills"]
# Per-unit flags: the FP64 set-up tables round like the reference's CPU model.
# The ray-marching kernels (atmo_rays.cu), the slab density kernel and the
# render-time queries use the approximate (<= 2 ulp) single-precision division
# and square root (the queries' lookups fall anywhere in the LUTs, and a
# 1920x1080 shading request takes 15% less time than with IEEE division); the
# transmittance and irradiance kernels keep IEEE division, whose exact results
# put lookups that start on LUT rows on texel centres and edges exactly where
# the reference does.
UNIT_FLAGS = {"atmo_tables.cu": ["--fmad=false"],
              "atmo_rays.cu": ["--prec-div=false", "--prec-sqrt=false"],
              "atmo_fast.cu": ["--prec-div=false", "--prec-sqrt=false"],
              "atmo_render.cu": ["--prec-div=false", "--prec-sqrt=false"]}
UNITS = ["atmo_tables.cu", "atmo_kernels.cu", "atmo_rays.cu", "atmo_fast.cu", "atmo_program.cu", "atmo_render.cu", "atmo_server.cu",
         "atmo_capi.cu", "atmo_noalloc.cu", "atmo_pass_api.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> str:
    build_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    extra = ["-DATMO_DEVICE_CHECKS"] if checked else []
    os.makedirs(build_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "atmo", "atmo.h"))
    objs, jobs = [], []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(build_dir, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers + [__file__]):
            cmd = [nvcc()] + ARCH + COMMON + extra + UNIT_FLAGS.get(u, []) + ["-c", src, "-o", obj]
            jobs.append(cmd)
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(lib, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        run(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, checked="--checked" in sys.argv))
