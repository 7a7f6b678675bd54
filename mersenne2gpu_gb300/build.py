"""Build recipe of the engine: libm2gpu.so (C ABI of include/m2gpu.h) and the
mersenne2 command line tool, compiled in-tree for sm_103a with nvcc.

Usage: python -m mersenne2gpu_gb300.build [--verbose] [--ptxas-info]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libm2gpu.so")
CLI = os.path.join(PKG, "mersenne2")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["m2_kernels.cu", "m2_rows.cu", "m2_cols.cu", "m2_carry.cu", "m2_api.cu", "m2_peaks.cu", "m2_noalloc.cu",
              "m2_gec.cu"]
CXX_SOURCES = ["m2_host.cpp"]
# the transform kernels, built a second time for the GF(P61^2)-only layout
# (-DM2_DUAL=0: namespace m2k_g61, the GF(P31^2) half compiled away)
GF61_SOURCES = ["m2_kernels.cu", "m2_rows.cu", "m2_cols.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str], verbose: bool) -> str:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout[-3000:]}\n{r.stderr[-6000:]}")
    return r.stdout + r.stderr


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h", ".inc"))]
    headers.append(os.path.join(ROOT, "include", "m2gpu.h"))
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", os.path.join(ROOT, "include")]
    jobs = []
    objs = []
    units = [(src, src + ".o", []) for src in CU_SOURCES] + [(src, src + ".g61.o", ["-DM2_DUAL=0"]) for src in GF61_SOURCES]
    for src, obj, defs in units:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        objs.append(o)
        cmd = [nv, *ARCH, "-lineinfo", *common, *defs, "--expt-relaxed-constexpr", "-c", s, "-o", o]
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
        if force or ptxas_info or _stale(o, [s, *headers]):
            jobs.append(cmd)
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", CSRC, "-c", s, "-o", o]
        if force or _stale(o, [s, *headers]):
            jobs.append(cmd)
    outputs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            outputs.append(out)
    if ptxas_info:
        for o in outputs:
            print(o)
    if force or jobs or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"], verbose)
    cli_src = os.path.join(CSRC, "mersenne2_cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB, os.path.join(ROOT, "include", "m2gpu.h")])):
        _run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-o", CLI, cli_src,
              "-I", "/usr/local/cuda/include", "-L", PKG, "-lm2gpu", "-L", "/usr/local/cuda/lib64", "-lcudart",
              f"-Wl,-rpath,{PKG}", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(verbose=a.verbose, ptxas_info=a.ptxas_info, force=a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
