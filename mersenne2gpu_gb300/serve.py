"""Serving loop on top of the engine's continuous-batching server (m2_srv_* in
include/m2gpu.h).

Requests arrive as a seeded Poisson stream with exponents log-uniform over the
primes in [1000, 18874367] (transform n = 32 ... 2^19).  The server admits
them while their device memory fits the budget, advances every admitted test
by a quantum of squarings per step (same-size small tests share one launch;
larger tests run on their own streams, concurrently), and retires finished
tests.  Reported per transform size: time-to-result p50/p99 over the requests
completed inside the window, the squarings done and the rate each test got
(completed and still active ones: a full test at n >= 4096 takes longer than
the window); overall: aggregate squarings/s, and a re-check of completed
results against the same tests run alone.
"""
from __future__ import annotations

import os

# Every three-pass test of the server runs on its own stream.  The CUDA driver
# maps streams onto CUDA_DEVICE_MAX_CONNECTIONS hardware work queues (8 unless
# set), and streams that share a queue serialise; 32, its largest value, let the
# tests' launches overlap (on a GB300: 130k -> 170k squarings/s in the 20 s
# seeded serving window).  It is read once, when the process first uses CUDA,
# so it is set here only if nothing has chosen it yet.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import ctypes  # noqa: E402
import statistics  # noqa: E402
import time  # noqa: E402
from dataclasses import dataclass  # noqa: E402

from . import MODE_PRP, Engine, _check, _lib  # noqa: E402
from .workloads import poisson_arrivals, serve_exponents  # noqa: E402


class _SrvResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("p", ctypes.c_uint32), ("mode", ctypes.c_int), ("iters", ctypes.c_uint32),
                ("res64", ctypes.c_uint64), ("is_prime", ctypes.c_int), ("status", ctypes.c_int),
                ("n", ctypes.c_uint64), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double),
                ("t_done", ctypes.c_double)]


class _SrvStats(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_uint32), ("active", ctypes.c_uint32), ("resident_bytes", ctypes.c_uint64),
                ("budget_bytes", ctypes.c_uint64), ("squarings", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("steps", ctypes.c_uint32), ("launches", ctypes.c_uint32)]


class _SrvProgress(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("p", ctypes.c_uint32), ("done", ctypes.c_uint32), ("total", ctypes.c_uint32),
                ("inflight", ctypes.c_uint32), ("n", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double)]


def _bind():
    L = _lib()
    if not getattr(L, "_m2_srv_bound", False):
        vp, u32, u64, i = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        L.m2_srv_create.argtypes = [ctypes.POINTER(vp), i, u64, u32]
        L.m2_srv_submit.argtypes = [vp, u64, u32, i, u32]
        L.m2_srv_step.argtypes = [vp]
        L.m2_srv_poll.argtypes = [vp, ctypes.POINTER(_SrvResult), i, ctypes.POINTER(i)]
        L.m2_srv_stats_get.argtypes = [vp, ctypes.POINTER(_SrvStats)]
        L.m2_srv_active_get.argtypes = [vp, ctypes.POINTER(_SrvProgress), i, ctypes.POINTER(i)]
        L.m2_srv_destroy.argtypes = [vp]
        L.m2_srv_destroy.restype = None
        for f in ("m2_srv_create", "m2_srv_submit", "m2_srv_step", "m2_srv_poll", "m2_srv_stats_get", "m2_srv_active_get"):
            getattr(L, f).restype = i
        L._m2_srv_bound = True
    return L


@dataclass
class Result:
    id: int
    p: int
    mode: int
    iters: int
    res64: int
    is_prime: bool
    status: int
    n: int
    t_submit: float
    t_admit: float
    t_done: float


class Server:
    """Continuous-batching server of independent tests on one GPU."""

    def __init__(self, budget_bytes: int, quantum: int = 1000, device: int = 0):
        self._L = _bind()
        self._h = ctypes.c_void_p()
        _check(self._L.m2_srv_create(ctypes.byref(self._h), device, budget_bytes, quantum), "m2_srv_create")

    def close(self) -> None:
        if self._h:
            self._L.m2_srv_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, rid: int, p: int, mode: int = MODE_PRP, iters: int = 0) -> None:
        _check(self._L.m2_srv_submit(self._h, rid, p, mode, iters), "m2_srv_submit")

    def step(self) -> None:
        _check(self._L.m2_srv_step(self._h), "m2_srv_step")

    def poll(self, max_results: int = 1024) -> list[Result]:
        arr = (_SrvResult * max_results)()
        n = ctypes.c_int()
        _check(self._L.m2_srv_poll(self._h, arr, max_results, ctypes.byref(n)), "m2_srv_poll")
        return [Result(a.id, a.p, a.mode, a.iters, a.res64, bool(a.is_prime), a.status, a.n, a.t_submit, a.t_admit,
                       a.t_done) for a in arr[: n.value]]

    def active(self, max_tests: int = 4096) -> list[dict]:
        """Progress of the admitted tests (admission order)."""
        arr = (_SrvProgress * max_tests)()
        n = ctypes.c_int()
        _check(self._L.m2_srv_active_get(self._h, arr, max_tests, ctypes.byref(n)), "m2_srv_active_get")
        return [{k: getattr(a, k) for k, _ in _SrvProgress._fields_} for a in arr[: n.value]]

    def stats(self) -> dict:
        s = _SrvStats()
        _check(self._L.m2_srv_stats_get(self._h, ctypes.byref(s)), "m2_srv_stats_get")
        return {k: getattr(s, k) for k, _ in _SrvStats._fields_}


def _pct(xs: list[float], q: float) -> float:
    xs = sorted(xs)
    if not xs:
        return float("nan")
    k = min(len(xs) - 1, max(0, int(round(q * (len(xs) - 1)))))
    return xs[k]


def run_serving(rate_per_s: float = 4.0, window_s: float = 20.0, budget_bytes: int = 8 << 30, quantum: int = 2000,
                n_requests: int = 2000, verify: int = 16, device: int = 0) -> dict:
    """Seeded Poisson stream of full PRP tests for `window_s` seconds; `verify`
    completed results (spread over the completion order) are re-run alone."""
    arrivals = poisson_arrivals(5, rate_per_s, n_requests)
    ps = serve_exponents(n_requests)
    done: list[Result] = []
    submitted = 0
    with Server(budget_bytes, quantum, device) as srv:
        t0 = time.perf_counter()
        sq0 = srv.stats()["squarings"]
        while True:
            now = time.perf_counter() - t0
            if now >= window_s:
                break
            while submitted < n_requests and arrivals[submitted] <= now:
                srv.submit(submitted, ps[submitted], MODE_PRP, 0)
                submitted += 1
            srv.step()
            done.extend(srv.poll())
            st = srv.stats()
            if st["active"] == 0 and st["queued"] == 0 and submitted < n_requests:
                time.sleep(max(0.0, min(0.01, arrivals[submitted] - (time.perf_counter() - t0))))
        elapsed = time.perf_counter() - t0
        st = srv.stats()
        squarings = st["squarings"] - sq0
        active = srv.active()
    # server clock at the end of the window: the latest time it reported, or the
    # host window (the server was created just before t0)
    t_end = max([elapsed] + [r.t_done for r in done])
    buckets: dict[int, dict] = {}
    for r in done:
        if r.status == 0:
            b = buckets.setdefault(r.n, {"lat": [], "rates": [], "squarings": 0, "active": 0})
            b["lat"].append(r.t_done - r.t_submit)
            b["rates"].append(r.iters / max(1e-9, r.t_done - r.t_admit))
            b["squarings"] += r.iters
    for a in active:
        b = buckets.setdefault(a["n"], {"lat": [], "rates": [], "squarings": 0, "active": 0})
        b["active"] += 1
        b["squarings"] += a["done"]
        if t_end > a["t_admit"]:
            b["rates"].append(a["done"] / (t_end - a["t_admit"]))
    per_n = {str(n): {"completed": len(b["lat"]), "p50_s": _pct(b["lat"], 0.50), "p99_s": _pct(b["lat"], 0.99),
                      "still_active": b["active"], "squarings": b["squarings"],
                      "squarings_per_s_per_test": statistics.fmean(b["rates"]) if b["rates"] else None}
             for n, b in sorted(buckets.items())}
    lat = [r.t_done - r.t_submit for r in done if r.status == 0]
    out = {
        "config": f"Poisson arrivals {rate_per_s}/s (seed 5), full PRP tests, p log-uniform over primes in "
                  f"[1000, 18874367], window {window_s:.0f} s, HBM budget {budget_bytes >> 20} MiB, "
                  f"quantum {quantum} squarings",
        "submitted": submitted, "completed": len(done), "errors": sum(1 for r in done if r.status != 0),
        "squarings_per_s": squarings / elapsed, "elapsed_s": elapsed, "p50_s": _pct(lat, 0.5), "p99_s": _pct(lat, 0.99),
        "per_n": per_n, "still_active": st["active"], "queued": st["queued"], "steps": st["steps"],
        "primes_found": sum(1 for r in done if r.is_prime),
    }
    if verify:
        ok = [r for r in done if r.status == 0]
        pick = ok[:: max(1, len(ok) // verify)][:verify] if ok else []
        same = 0
        for r in pick:
            with Engine(r.p, r.mode, device=device) as e:
                e.iterate(r.iters)
                same += int(e.res64() == r.res64 and e.verdict() == r.is_prime)
        out["bit_exact_vs_alone"] = f"{same}/{len(pick)} re-run alone"
    return out
