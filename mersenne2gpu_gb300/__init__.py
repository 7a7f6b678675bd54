"""GB300-native Lucas-Lehmer / PRP engine for Mersenne numbers 2^p - 1.

Python binding of the C ABI in include/m2gpu.h (libm2gpu.so, built in-tree by
mersenne2gpu_gb300.build).  There is no CPU fallback: every call runs the CUDA
kernels, and importing the binding raises if the library was not built.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libm2gpu.so")

MODE_LL, MODE_PRP, MODE_PRP3 = 0, 1, 2
PATH_AUTO, PATH_SMALL, PATH_LARGE = 0, 1, 2
FIELDS_DUAL, FIELDS_GF61 = 0, 1
_MODES = {"ll": MODE_LL, "prp": MODE_PRP, "prp3": MODE_PRP3}

# every symbol include/m2gpu.h declares
EXPORTS = (
    "m2_create", "m2_iterate", "m2_sync", "m2_get_digits", "m2_set_digits", "m2_res64",
    "m2_verdict", "m2_info", "m2_destroy", "m2_layout", "m2_strerror", "m2_batch_run",
    "m2_profile", "m2_launches_for", "m2_measure_mul_peak", "m2_square_noalloc",
    "m2_srv_create", "m2_srv_submit", "m2_srv_step", "m2_srv_poll", "m2_srv_stats_get", "m2_srv_active_get",
    "m2_srv_destroy",
    "m2_last_error", "m2_carry_normalize", "m2_batch_tuned", "m2_batch_tuning", "m2_layout_fields", "m2_test_stall_fused",
    "m2_test_stage",
    "m2_gec_create", "m2_gec_iterate", "m2_gec_check", "m2_gec_verified", "m2_gec_stats_get", "m2_gec_destroy",
)
E_CHECK = -7   # M2_ECHECK


class M2Error(RuntimeError):
    def __init__(self, code: int, what: str):
        detail = _lib().m2_last_error().decode() if code in (-2, -3) else ""
        super().__init__(f"{what}: {_lib().m2_strerror(code).decode()} ({code})" + (f" [{detail}]" if detail else ""))
        self.code = code


class _Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("wg", ctypes.c_uint32), ("carry_pairs", ctypes.c_uint32),
                ("path", ctypes.c_int), ("stream", ctypes.c_void_p), ("fields", ctypes.c_int),
                ("fused_middle", ctypes.c_int)]


class _Info(ctypes.Structure):
    _fields_ = [("p", ctypes.c_uint32), ("mode", ctypes.c_int), ("ln", ctypes.c_int), ("n", ctypes.c_uint64),
                ("iteration", ctypes.c_uint32), ("total_iters", ctypes.c_uint32), ("path", ctypes.c_int),
                ("rows", ctypes.c_uint32), ("row_len", ctypes.c_uint32), ("cols_per_cta", ctypes.c_uint32),
                ("span", ctypes.c_uint32), ("device_bytes", ctypes.c_uint64), ("fused_cols", ctypes.c_uint32),
                ("fields", ctypes.c_int)]


class _StageTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("ms_per_launch", ctypes.c_double), ("launches", ctypes.c_uint64),
                ("bytes_per_launch", ctypes.c_uint64), ("iters_per_launch", ctypes.c_uint32)]


class _GecStats(ctypes.Structure):
    _fields_ = [("verified_iter", ctypes.c_uint32), ("block", ctypes.c_uint32), ("updates", ctypes.c_uint64),
                ("checks", ctypes.c_uint64), ("failures", ctypes.c_uint64), ("seconds", ctypes.c_double)]


class _BatchTuning(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int), ("carry_blocks", ctypes.c_int), ("carry_pairs", ctypes.c_int),
                ("fused_middle", ctypes.c_int), ("ns_per_test_iter", ctypes.c_double), ("ns_default", ctypes.c_double)]


class _BatchStats(ctypes.Structure):
    _fields_ = [("seconds", ctypes.c_double), ("squarings", ctypes.c_uint64), ("launches", ctypes.c_uint32),
                ("buckets", ctypes.c_uint32)]


_LIB = None


def _lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run `python -m mersenne2gpu_gb300.build` first")
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, i = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        L.m2_create.argtypes = [ctypes.POINTER(vp), u32, i, ctypes.POINTER(_Opts)]
        L.m2_iterate.argtypes = [vp, u32]
        L.m2_sync.argtypes = [vp]
        L.m2_get_digits.argtypes = [vp, vp]
        L.m2_set_digits.argtypes = [vp, vp, u32]
        L.m2_res64.argtypes = [vp, ctypes.POINTER(u64)]
        L.m2_verdict.argtypes = [vp, ctypes.POINTER(i)]
        L.m2_info.argtypes = [vp, ctypes.POINTER(_Info)]
        L.m2_destroy.argtypes = [vp]
        L.m2_destroy.restype = None
        L.m2_layout.argtypes = [u32, ctypes.POINTER(i), ctypes.POINTER(u64), vp]
        L.m2_layout_fields.argtypes = [u32, i, ctypes.POINTER(i), ctypes.POINTER(u64), vp]
        L.m2_strerror.argtypes = [i]
        L.m2_strerror.restype = ctypes.c_char_p
        L.m2_batch_run.argtypes = [vp, vp, vp, ctypes.c_size_t, vp, vp, i, ctypes.POINTER(_BatchStats)]
        L.m2_profile.argtypes = [vp, u32, ctypes.POINTER(_StageTime), i, ctypes.POINTER(i)]
        L.m2_launches_for.argtypes = [vp, u32]
        L.m2_launches_for.restype = u64
        L.m2_measure_mul_peak.argtypes = [i, ctypes.POINTER(ctypes.c_double)]
        L.m2_square_noalloc.argtypes = [u32, i, vp, u32, vp]
        L.m2_carry_normalize.argtypes = [u32, vp, vp, u32, vp, vp]
        L.m2_test_stall_fused.argtypes = [vp]
        L.m2_test_stage.argtypes = [vp, i, vp, vp]
        L.m2_batch_tuned.argtypes = [i, i, ctypes.POINTER(i), ctypes.POINTER(ctypes.c_double)]
        L.m2_batch_tuning.argtypes = [i, i, ctypes.POINTER(_BatchTuning)]
        L.m2_last_error.argtypes = []
        L.m2_gec_create.argtypes = [ctypes.POINTER(vp), vp, u32]
        L.m2_gec_iterate.argtypes = [vp, u32]
        L.m2_gec_check.argtypes = [vp, ctypes.POINTER(u32)]
        L.m2_gec_verified.argtypes = [vp, vp, ctypes.POINTER(u32)]
        L.m2_gec_stats_get.argtypes = [vp, ctypes.POINTER(_GecStats)]
        L.m2_gec_destroy.argtypes = [vp]
        L.m2_last_error.restype = ctypes.c_char_p
        for name in EXPORTS:
            if name not in ("m2_destroy", "m2_strerror", "m2_launches_for", "m2_last_error", "m2_gec_destroy") \
                    and not name.startswith("m2_srv"):
                getattr(L, name).restype = i
        _LIB = L
    return _LIB


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise M2Error(rc, what)


def layout(p: int, fields: int = FIELDS_DUAL) -> tuple[int, int, np.ndarray]:
    """(log2 n, n, digit widths) of exponent p for a field set; no device needed."""
    L = _lib()
    ln, n = ctypes.c_int(), ctypes.c_uint64()
    _check(L.m2_layout_fields(p, fields, ctypes.byref(ln), ctypes.byref(n), None), "m2_layout_fields")
    w = np.zeros(n.value, dtype=np.uint8)
    _check(L.m2_layout_fields(p, fields, ctypes.byref(ln), ctypes.byref(n), w.ctypes.data), "m2_layout_fields")
    return ln.value, n.value, w


def total_iterations(p: int, mode: int) -> int:
    return {MODE_LL: p - 2, MODE_PRP: p, MODE_PRP3: p - 1}[mode]


@dataclass
class Info:
    p: int
    mode: int
    ln: int
    n: int
    iteration: int
    total_iters: int
    path: int
    rows: int
    row_len: int
    cols_per_cta: int
    span: int
    device_bytes: int
    fused_cols: int
    fields: int


class Engine:
    """One test of 2^p - 1 on one GPU (wraps an m2_ctx)."""

    def __init__(self, p: int, mode: int | str = MODE_PRP, device: int = 0, path: int = PATH_AUTO,
                 wg: int = 0, carry_pairs: int = 0, stream: int | None = None, fields: int = FIELDS_DUAL,
                 fused_middle: int = 0):
        if isinstance(mode, str):
            mode = _MODES[mode.lower()]
        self._L = _lib()
        self._h = ctypes.c_void_p()
        o = _Opts(device, wg, carry_pairs, path, stream, fields, fused_middle)
        _check(self._L.m2_create(ctypes.byref(self._h), p, mode, ctypes.byref(o)), f"m2_create(p={p})")
        self.p, self.mode = p, mode
        self.info()

    def close(self) -> None:
        if self._h:
            self._L.m2_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> Info:
        i = _Info()
        _check(self._L.m2_info(self._h, ctypes.byref(i)), "m2_info")
        self.n = i.n
        return Info(i.p, i.mode, i.ln, i.n, i.iteration, i.total_iters, i.path, i.rows, i.row_len,
                    i.cols_per_cta, i.span, i.device_bytes, i.fused_cols, i.fields)

    def iterate(self, k: int) -> None:
        _check(self._L.m2_iterate(self._h, k), "m2_iterate")

    def sync(self) -> None:
        _check(self._L.m2_sync(self._h), "m2_sync")

    def digits(self, out: np.ndarray | None = None) -> np.ndarray:
        """Canonical digits; `out` (n uint64, contiguous, e.g. a view of pinned
        host memory, which the copy then reaches by DMA) is filled if given."""
        if out is None:
            out = np.zeros(self.n, dtype=np.uint64)
        elif out.dtype != np.uint64 or out.shape != (self.n,) or not out.flags.c_contiguous:
            raise ValueError(f"expected a contiguous uint64 array of {self.n} digits")
        _check(self._L.m2_get_digits(self._h, out.ctypes.data), "m2_get_digits")
        return out

    def set_digits(self, d: np.ndarray, iteration: int) -> None:
        d = np.ascontiguousarray(d, dtype=np.uint64)
        if d.shape != (self.n,):
            raise ValueError(f"expected {self.n} digits")
        _check(self._L.m2_set_digits(self._h, d.ctypes.data, iteration), "m2_set_digits")

    def res64(self) -> int:
        r = ctypes.c_uint64()
        _check(self._L.m2_res64(self._h, ctypes.byref(r)), "m2_res64")
        return r.value

    def verdict(self) -> bool:
        v = ctypes.c_int()
        _check(self._L.m2_verdict(self._h, ctypes.byref(v)), "m2_verdict")
        return bool(v.value)

    def test_stage(self, stage: int) -> tuple[np.ndarray, np.ndarray]:
        """Runs one stage of a squaring (three-pass path; m2_test_stage) and
        returns the transform elements it leaves: (h, 2) uint64 GF(P61^2) and
        (h, 2) uint32 GF(P31^2) coordinates, element r B + c."""
        h = self.n // 2
        za = np.zeros((h, 2), dtype=np.uint64)
        zb = np.zeros((h, 2), dtype=np.uint32)
        _check(self._L.m2_test_stage(self._h, stage, za.ctypes.data, zb.ctypes.data), f"m2_test_stage({stage})")
        return za, zb

    def profile(self, iters: int) -> list[dict]:
        """Per-stage average device time over `iters` squarings (advances the state)."""
        arr = (_StageTime * 8)()
        cnt = ctypes.c_int()
        _check(self._L.m2_profile(self._h, iters, arr, 8, ctypes.byref(cnt)), "m2_profile")
        return [dict(name=a.name.decode(), ms_per_launch=a.ms_per_launch, launches=a.launches,
                     bytes_per_launch=a.bytes_per_launch, iters_per_launch=a.iters_per_launch)
                for a in arr[: cnt.value]]

    def launches_for(self, k: int) -> int:
        return int(self._L.m2_launches_for(self._h, k))

    def run(self) -> bool:
        """Remaining iterations to completion; returns the verdict."""
        i = self.info()
        self.iterate(i.total_iters - i.iteration)
        return self.verdict()


class Gec:
    """Gerbicz error check of an Engine's PRP chain (wraps an m2_gec).

    iterate(k) advances the engine by k squarings and updates the check product
    every `block` squarings; check() verifies everything since the last
    verified state and returns True, or returns False after putting the engine
    back to that state (its iteration is then `verified_iter`)."""

    def __init__(self, engine: Engine, block: int):
        self._L = engine._L
        self.engine = engine
        self._h = ctypes.c_void_p()
        _check(self._L.m2_gec_create(ctypes.byref(self._h), engine._h, block), f"m2_gec_create(block={block})")
        self.verified_iter = engine.info().iteration

    def close(self) -> None:
        if self._h:
            self._L.m2_gec_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def iterate(self, k: int) -> None:
        _check(self._L.m2_gec_iterate(self._h, k), "m2_gec_iterate")

    def check(self) -> bool:
        v = ctypes.c_uint32()
        rc = self._L.m2_gec_check(self._h, ctypes.byref(v))
        self.verified_iter = v.value
        if rc == E_CHECK:
            return False
        _check(rc, "m2_gec_check")
        return True

    def verified(self) -> tuple[np.ndarray, int]:
        d = np.zeros(self.engine.n, dtype=np.uint64)
        it = ctypes.c_uint32()
        _check(self._L.m2_gec_verified(self._h, d.ctypes.data, ctypes.byref(it)), "m2_gec_verified")
        return d, it.value

    def stats(self) -> dict:
        st = _GecStats()
        _check(self._L.m2_gec_stats_get(self._h, ctypes.byref(st)), "m2_gec_stats_get")
        return {k: getattr(st, k) for k, _ in _GecStats._fields_}


def measure_mul_peak(device: int = 0) -> float:
    """Peak 32x32->64-bit integer products per second on the device."""
    r = ctypes.c_double()
    _check(_lib().m2_measure_mul_peak(device, ctypes.byref(r)), "m2_measure_mul_peak")
    return r.value


@dataclass
class BatchResult:
    res64: np.ndarray
    is_prime: np.ndarray
    seconds: float
    squarings: int
    launches: int
    buckets: int


def batch_run(ps, modes=None, iters=None, device: int = 0) -> BatchResult:
    """Independent tests in bucketed persistent launches (m2_batch_run)."""
    L = _lib()
    p = np.ascontiguousarray(ps, dtype=np.uint32)
    cnt = len(p)
    m = None if modes is None else np.ascontiguousarray(
        [(_MODES[x] if isinstance(x, str) else x) for x in modes], dtype=np.int32)
    it = None if iters is None else np.ascontiguousarray(iters, dtype=np.uint32)
    res = np.zeros(cnt, dtype=np.uint64)
    pr = np.zeros(cnt, dtype=np.int32)
    st = _BatchStats()
    _check(L.m2_batch_run(p.ctypes.data, None if m is None else m.ctypes.data, None if it is None else it.ctypes.data,
                          cnt, res.ctypes.data, pr.ctypes.data, device, ctypes.byref(st)), "m2_batch_run")
    return BatchResult(res, pr.astype(bool), st.seconds, st.squarings, st.launches, st.buckets)


def carry_normalize(p: int, digits, carries=None, seg: int = 0, out=None, stream=None):
    """Full carry propagation on the device (m2_carry_normalize): `digits` (and
    `carries`) are int64 CUDA tensors of exponent p's layout; returns the n
    canonical digits as a uint64-valued int64 CUDA tensor (`out` if given)."""
    import torch
    L = _lib()
    n = len(digits)
    if out is None:
        out = torch.empty(n, dtype=torch.int64, device=digits.device)
    s = torch.cuda.current_stream(digits.device).cuda_stream if stream is None else stream
    _check(L.m2_carry_normalize(p, digits.data_ptr(), None if carries is None else carries.data_ptr(), seg,
                                out.data_ptr(), s), "m2_carry_normalize")
    return out


def batch_tuned(ln: int, device: int = 0) -> tuple[int, float] | None:
    """(threads per transform, ns per test-squaring) m2_batch_run chose for n = 2^ln."""
    t, ns = ctypes.c_int(), ctypes.c_double()
    rc = _lib().m2_batch_tuned(device, ln, ctypes.byref(t), ctypes.byref(ns))
    return (t.value, ns.value) if rc == 0 else None


def batch_tuning(ln: int, device: int = 0) -> dict | None:
    """The batch autotuner's choice for transform size 2^ln (None if not tuned):
    threads per transform, carry blocks and their length in digit pairs (-B),
    fused or separate transform middle, and the measured ns per test-squaring
    of the choice and of the untuned default."""
    t = _BatchTuning()
    if _lib().m2_batch_tuning(device, ln, ctypes.byref(t)) != 0:
        return None
    return {"threads": t.threads, "carry_blocks": t.carry_blocks, "carry_pairs": t.carry_pairs,
            "fused_middle": t.fused_middle, "ns_per_test_squaring": t.ns_per_test_iter,
            "ns_default": t.ns_default}
