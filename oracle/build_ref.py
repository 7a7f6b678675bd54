"""Build the CPU oracles (test infrastructure only).

1. oracle/m2_oracle.c (the plain-C restatement) -> oracle/_build/liboracle.so
2. the reference's own kernels -> oracle/_ref/libm2ref.so (for the CPU):
   when the reference checkout is present, the host math (mersenne2_gpu.cpp:75-293)
   and the OpenCL kernel string KC (mersenne2_gpu.cpp:295-3026) are cut out of
   it, by marker, into oracle/_ref/ref_host.inc and oracle/_ref/ref_kernels.inc
   (git-ignored; the reference sources are never committed), then
   oracle/ref_driver.cpp is compiled against them.  Where the checkout is
   absent but the .inc files are there (a copy of this tree taken elsewhere),
   only the compile step runs.
3. the reference program itself, OpenCL host code and all (mersenne2_gpu.cpp,
   copied whole into oracle/_ref/) -> oracle/_ref/mersenne2_ocl, compiled
   against the hand-declared OpenCL prototypes of oracle/ocl_min/CL/cl.h and
   the minimal ICD dispatcher oracle/ocl_min/icd_min.cpp, which reaches the
   vendor's OpenCL driver at run time (oracle.ref_opencl_run).  It times the
   reference's own GPU path; building it needs no GPU.

Usage: python oracle/build_ref.py [--reference DIR]
The reference checkout is DIR, else $M2_REFERENCE, else a directory named
"reference" beside this repository.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BUILD_DIR = os.path.join(HERE, "_build")
DEFAULT_REFERENCE = os.environ.get("M2_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def extract(reference: str) -> bool:
    src = os.path.join(reference, "mersenne2_gpu.cpp")
    if not os.path.isfile(src):
        return False
    text = open(src, encoding="utf-8").read()
    os.makedirs(REF_DIR, exist_ok=True)
    with open(os.path.join(REF_DIR, "mersenne2_gpu.cpp"), "w", encoding="utf-8") as f:
        f.write(text)
    host_begin = text.index("static const uint64_t Z61_p")
    kc_decl = text.index('const char* KC = R"CLC(')
    kc_begin = kc_decl + len('const char* KC = R"CLC(')
    kc_end = text.index(')CLC";', kc_begin)
    os.makedirs(REF_DIR, exist_ok=True)
    with open(os.path.join(REF_DIR, "ref_host.inc"), "w", encoding="utf-8") as f:
        f.write("// generated by oracle/build_ref.py from the reference checkout; not committed\n")
        f.write("#include <vector>\n#include <cstdint>\n")
        f.write(text[host_begin:kc_decl])
    with open(os.path.join(REF_DIR, "ref_kernels.inc"), "w", encoding="utf-8") as f:
        f.write("// generated by oracle/build_ref.py from the reference checkout; not committed\n")
        f.write(text[kc_begin:kc_end])
    return True


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)} failed:\n{r.stderr[-4000:]}")


def build_oracle() -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    out = os.path.join(BUILD_DIR, "liboracle.so")
    src = os.path.join(HERE, "m2_oracle.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        _run(["gcc", "-O2", "-shared", "-fPIC", "-o", out, src])
    return out


def build_ref(reference: str = DEFAULT_REFERENCE) -> str | None:
    extract(reference)
    inc = [os.path.join(REF_DIR, f) for f in ("ref_host.inc", "ref_kernels.inc")]
    if not all(os.path.isfile(p) for p in inc):
        return None
    out = os.path.join(REF_DIR, "libm2ref.so")
    src = os.path.join(HERE, "ref_driver.cpp")
    deps = inc + [src, os.path.join(HERE, "ref_shim.hpp")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    base = ["g++", "-O2", "-std=c++20", "-shared", "-fPIC", "-w", "-I", HERE, "-o", out, src]
    try:
        _run(base[:1] + ["-fopenmp"] + base[1:])
    except RuntimeError:
        _run(base)  # no OpenMP runtime: single-threaded build
    return out


def build_ref_opencl(reference: str = DEFAULT_REFERENCE) -> str | None:
    """The reference program with its OpenCL host path (None without its source)."""
    extract(reference)
    src = os.path.join(REF_DIR, "mersenne2_gpu.cpp")
    if not os.path.isfile(src):
        return None
    out = os.path.join(REF_DIR, "mersenne2_ocl")
    ocl = os.path.join(HERE, "ocl_min")
    deps = [src, os.path.join(ocl, "CL", "cl.h"), os.path.join(ocl, "icd_min.cpp")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    _run(["g++", "-O2", "-std=c++20", "-w", "-I", ocl, "-o", out, src, os.path.join(ocl, "icd_min.cpp"), "-ldl"])
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    a = ap.parse_args()
    print(build_oracle())
    print(build_ref(a.reference))
    print(build_ref_opencl(a.reference))
    return 0


if __name__ == "__main__":
    sys.exit(main())
