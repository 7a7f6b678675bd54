"""CPU oracles of the squaring chain -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
arm may import this package, and only as the checker (or as the timed CPU
baseline).  The product (mersenne2gpu_gb300, libm2gpu.so, the mersenne2 CLI)
never imports, links or calls it.

* Oracle      -- oracle/m2_oracle.c, a plain-C restatement of the reference's
                 algorithm (mersenne2_gpu.cpp; see the file header for the
                 per-function line citations).
* RefKernels  -- the reference's own OpenCL C kernels compiled for the CPU
                 (oracle/ref_driver.cpp + oracle/build_ref.py), run in the
                 order of its generic launch plan.
* python_chain -- exact Python-integer chain for small cases.
* ref_opencl_run -- the reference program itself on the GPU through the
                 vendor's OpenCL driver, where one is installed: the timing of
                 the reference's own GPU path, never a checker of this
                 engine's digits.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_ref as _build

HERE = os.path.dirname(os.path.abspath(__file__))
LL, PRP, PRP3 = 0, 1, 2


def build(reference: str = _build.DEFAULT_REFERENCE) -> tuple[str, str | None]:
    out = _build.build_oracle(), _build.build_ref(reference)
    try:
        _build.build_ref_opencl(reference)
    except RuntimeError:
        pass   # the reference program only serves timing; the CPU oracles above do not depend on it
    return out


# where NVIDIA's driver installs its OpenCL implementation
_OPENCL_VENDOR_LIBS = ("/usr/lib/libnvidia-opencl.so.1", "/usr/lib64/libnvidia-opencl.so.1",
                       "/usr/lib/aarch64-linux-gnu/libnvidia-opencl.so.1",
                       "/usr/lib/x86_64-linux-gnu/libnvidia-opencl.so.1",
                       "/usr/local/nvidia/lib64/libnvidia-opencl.so.1")


def opencl_vendor_lib() -> str | None:
    for c in _OPENCL_VENDOR_LIBS:
        if os.path.exists(c):
            return c
    return None


def ref_opencl_run(args: list[str], timeout: float = 600.0) -> tuple[int, str]:
    """Runs the reference program (oracle/_ref/mersenne2_ocl) with its own
    argv `args` on the GPU through the vendor OpenCL driver; returns (exit
    code, stdout + stderr).  RuntimeError when the program or a driver is
    missing."""
    import subprocess
    exe = _build.build_ref_opencl()
    if exe is None:
        raise RuntimeError("reference program not built (reference source absent)")
    vend = opencl_vendor_lib()
    if vend is None:
        raise RuntimeError("no vendor OpenCL driver library on this machine")
    env = dict(os.environ, M2_OCL_VENDOR_LIB=vend)
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=timeout, env=env)
    return r.returncode, r.stdout + r.stderr


_O = None
_R = None


def _oracle_lib() -> ctypes.CDLL:
    global _O
    if _O is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.o_create.restype = vp
        L.o_create.argtypes = [ctypes.c_uint32, ctypes.c_int]
        L.o_destroy.argtypes = [vp]
        L.o_iterate.argtypes = [vp, ctypes.c_uint32]
        L.o_n.restype = ctypes.c_uint64
        L.o_n.argtypes = [vp]
        L.o_ln.argtypes = [vp]
        L.o_get_digits.argtypes = [vp, vp]
        L.o_set_digits.argtypes = [vp, vp, ctypes.c_uint32]
        L.o_widths.argtypes = [vp, vp]
        L.o_shifts.argtypes = [vp, vp, vp]
        L.o_twiddles.argtypes = [vp, vp]
        L.o_res64.restype = ctypes.c_uint64
        L.o_res64.argtypes = [vp]
        L.o_verdict.argtypes = [vp]
        L.o_transformsize.argtypes = [ctypes.c_uint64]
        _O = L
    return _O


def transformsize(p: int) -> int:
    return _oracle_lib().o_transformsize(p)


class Oracle:
    """The C restatement of one test (state = canonical digits)."""

    def __init__(self, p: int, mode: int):
        self._L = _oracle_lib()
        self._h = self._L.o_create(p, mode)
        if not self._h:
            raise ValueError(f"oracle: bad p={p} / mode={mode}")
        self.p, self.mode = p, mode
        self.n = int(self._L.o_n(self._h))
        self.ln = int(self._L.o_ln(self._h))

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.o_destroy(self._h)
            self._h = None

    def iterate(self, k: int) -> None:
        self._L.o_iterate(self._h, k)

    def digits(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.uint64)
        self._L.o_get_digits(self._h, out.ctypes.data)
        return out

    def set_digits(self, d: np.ndarray, iteration: int) -> None:
        d = np.ascontiguousarray(d, dtype=np.uint64)
        self._L.o_set_digits(self._h, d.ctypes.data, iteration)

    def widths(self) -> np.ndarray:
        w = np.zeros(self.n, dtype=np.uint8)
        self._L.o_widths(self._h, w.ctypes.data)
        return w

    def shifts(self) -> tuple[np.ndarray, np.ndarray]:
        a = np.zeros(self.n, dtype=np.uint8)
        b = np.zeros(self.n, dtype=np.uint8)
        self._L.o_shifts(self._h, a.ctypes.data, b.ctypes.data)
        return a, b

    def res64(self) -> int:
        return int(self._L.o_res64(self._h))

    def verdict(self) -> bool:
        return bool(self._L.o_verdict(self._h))


def _ref_lib() -> ctypes.CDLL | None:
    global _R
    if _R is None:
        path = _build.build_ref()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.ref_create.restype = vp
        L.ref_create.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32]
        L.ref_destroy.argtypes = [vp]
        L.ref_iterate.argtypes = [vp, ctypes.c_uint32]
        L.ref_get_digits.argtypes = [vp, vp]
        L.ref_n.restype = ctypes.c_uint64
        L.ref_n.argtypes = [vp]
        _R = L
    return _R


def ref_available() -> bool:
    try:
        return _ref_lib() is not None
    except Exception:
        return False


class RefKernels:
    """The reference's own kernels on the host (LL / PRP only)."""

    def __init__(self, p: int, mode: int, carry_pairs: int = 64):
        L = _ref_lib()
        if L is None:
            raise RuntimeError("reference kernels not built (reference checkout absent)")
        self._L = L
        self._h = L.ref_create(p, mode, carry_pairs)
        if not self._h:
            raise ValueError(f"reference: bad p={p} / mode={mode}")
        self.n = int(L.ref_n(self._h))

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.ref_destroy(self._h)
            self._h = None

    def iterate(self, k: int) -> None:
        self._L.ref_iterate(self._h, k)

    def digits(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.uint64)
        self._L.ref_get_digits(self._h, out.ctypes.data)
        return out

    @staticmethod
    def threads() -> int:
        L = _ref_lib()
        return int(L.ref_threads()) if L is not None else 0

    @staticmethod
    def set_threads(n: int) -> None:
        """Threads of the work-item loops from now on (OpenMP)."""
        L = _ref_lib()
        if L is not None:
            L.ref_set_threads(ctypes.c_int(n))


def python_chain(p: int, mode: int, iters: int, x0: int | None = None) -> int:
    """Exact x after `iters` steps (Python integers); small p only."""
    M = (1 << p) - 1
    x = x0 if x0 is not None else (4 if mode == LL else 3)
    for _ in range(iters):
        if mode == LL:
            x = (x * x - 2) % M
        elif mode == PRP:
            x = (x * x) % M
        else:
            x = (3 * x * x) % M
    return x


def value_of_digits(digits: np.ndarray, widths: np.ndarray) -> int:
    v, pos = 0, 0
    for d, w in zip(digits.tolist(), widths.tolist()):
        v |= int(d) << pos
        pos += int(w)
    return v


def digits_of_value(v: int, widths: np.ndarray) -> np.ndarray:
    out = np.zeros(len(widths), dtype=np.uint64)
    for j, w in enumerate(widths.tolist()):
        out[j] = v & ((1 << int(w)) - 1)
        v >>= int(w)
    return out
