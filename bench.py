#!/usr/bin/env python3
"""Benchmark of the GB300 Lucas-Lehmer / PRP engine.

Headline: ms per squaring iteration of the PRP test of p = 57885161 (transform
n = 2^21 digits, 25 MB of dual-field state), the configuration the reference's
README lists as its large example (README.md:58).  A "step" is one report batch
of --iters-per-step squarings (the reference synchronises once per report batch,
mersenne2_gpu.cpp:4803-4853); L2 is flushed (a 256 MB write, larger than the
129 MB L2) between timed steps, outside the CUDA events.

Also reported:
  e2e       the same metric through the C ABI with host buffers: every step
            uploads the digits (m2_set_digits), iterates, and reads the
            canonical digits back (m2_get_digits), copies inside the timed region
  roofline  the dominant kernel's algorithmic bytes / CUDA-event time against
            the measured HBM copy bandwidth; roofline_imad: integer-product
            count against the measured mad.wide.u32 peak
  cpu_baseline  the reference's own kernels on the host cores (oracle/_ref),
            bounded sample
  reference_opencl_gpu  the reference program itself (mersenne2_gpu.cpp, its
            OpenCL host code and kernels) on this GPU through the vendor
            OpenCL driver: ms/iter from its own progress lines
  batched   config "4096 seeded PRP tests, p in [3, 159739]" through the batched
            engine vs one test at a time (sampled), res64 bit-exact
  serving   seeded Poisson stream of PRP requests, p log-uniform in
            [1000, 18874367], continuous batching under an HBM budget for a
            fixed window: p50/p99 time-to-result per transform size,
            squarings/s, completed results re-run alone
  parity    res64 against GMP's at every step boundary that is a golden
            checkpoint (every 1000 squarings up to 30000 at n = 2^21; 20000 at
            n = 2^22), read between the timed intervals

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

# the serving leg runs each large test on its own stream: 32 hardware work
# queues (not the default 8) let them overlap; read when CUDA starts
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
# the CPU rows (the reference's kernels under OpenMP) pin one thread per core,
# in both arms, so that their figures are comparable
os.environ.setdefault("OMP_PROC_BIND", "close")
os.environ.setdefault("OMP_PLACES", "cores")

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DEFAULT_P = 57885161
WORKLOAD = "PRP p=57885161 (n=2^21 digits, h=2^20 dual-field elements)"
METRIC = "ms/iter at N=2^21 (p=57885161)"
GOLDEN_LARGE = os.path.join(ROOT, "tests", "golden", "large.json")
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "traffic.json")
L2_FLUSH_BYTES = 256 << 20


def _env_int(k: str, d: int) -> int:
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class Dist:
    def __init__(self):
        self.world = _env_int("WORLD_SIZE", 1)
        self.rank = _env_int("RANK", 0)
        self.local = _env_int("LOCAL_RANK", 0)
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "nccl" if _cuda_ok() else "gloo"
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg is not None:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if self.pg is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if _cuda_ok() else "cpu")
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg is not None:
            self.pg.destroy_process_group()


def _cuda_ok() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def _load_json(path: str):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def wide_mul_count(h: int) -> int:
    """32x32->64-bit products of one squaring: 15 per dual-field GF multiplication,
    G(h) = 0.75 h log2 h + 2 h GF multiplications (forward + inverse radix-4 + centre)."""
    lg = h.bit_length() - 1
    return int(15 * (0.75 * h * lg + 2 * h))


# ---------------------------------------------------------------- reference arm
def reference_sample(p: int, iters: int) -> tuple[float, int, float]:
    """(ms per iteration, threads, setup seconds) of the reference's own kernels on the host."""
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    r = oracle.RefKernels(p, oracle.PRP)
    setup = time.perf_counter() - t0
    r.iterate(1)
    t0 = time.perf_counter()
    r.iterate(iters)
    dt = time.perf_counter() - t0
    return dt / iters * 1e3, oracle.RefKernels.threads(), setup


def reference_single_thread(p: int, iters: int) -> float:
    """ms per iteration of the reference's own kernels on one host thread."""
    import oracle
    all_threads = oracle.RefKernels.threads()
    r = oracle.RefKernels(p, oracle.PRP)
    try:
        oracle.RefKernels.set_threads(1)
        r.iterate(1)
        t0 = time.perf_counter()
        r.iterate(iters)
        return (time.perf_counter() - t0) / iters * 1e3
    finally:
        oracle.RefKernels.set_threads(all_threads)


def gmp_sample(p: int, iters: int) -> dict:
    """Single-thread GMP (mpz_mul, then the fold mod 2^p - 1) on a full-size
    residue: a secondary CPU row beside the reference's own kernels."""
    import ctypes
    import ctypes.util
    G = ctypes.CDLL(ctypes.util.find_library("gmp") or "libgmp.so.10")

    class Z(ctypes.Structure):
        _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]

    x, m, hi = Z(), Z(), Z()
    bx, bm, bh = ctypes.byref(x), ctypes.byref(m), ctypes.byref(hi)
    ul = ctypes.c_ulong
    for z in (bx, bm, bh):
        G.__gmpz_init(z)
    try:
        G.__gmpz_ui_pow_ui(bm, ul(2), ul(p))
        G.__gmpz_sub_ui(bm, bm, ul(1))            # M_p
        G.__gmpz_tdiv_q_ui(bx, bm, ul(3))         # a full-size residue (M_p - 12345 would square to a tiny one)

        def square():
            G.__gmpz_mul(bx, bx, bx)
            G.__gmpz_tdiv_q_2exp(bh, bx, ul(p))
            G.__gmpz_tdiv_r_2exp(bx, bx, ul(p))
            G.__gmpz_add(bx, bx, bh)
            if G.__gmpz_cmp(bx, bm) >= 0:
                G.__gmpz_sub(bx, bx, bm)

        square()
        t0 = time.perf_counter()
        for _ in range(iters):
            square()
        ms = (time.perf_counter() - t0) / iters * 1e3
        G.__gmpz_sizeinbase.restype = ctypes.c_size_t
        bits = int(G.__gmpz_sizeinbase(bx, 2))
        if bits < p - 64:
            raise RuntimeError(f"residue shrank to {bits} bits")
    finally:
        for z in (bx, bm, bh):
            G.__gmpz_clear(z)
    return {"value": ms, "unit": "ms/iter", "cores": 1, "kind": "gmp",
            "sample": f"{iters} squarings mod 2^{p}-1 of a full-size residue with libgmp mpz_mul (one thread)"}


def run_reference(a, dist: Dist) -> dict | None:
    if dist.rank != 0:
        return None
    import oracle
    if not oracle.ref_available():
        return {"impl": "reference", "unavailable": "reference kernel sources not extracted (oracle/_ref missing)"}
    oracle.build()
    r = oracle.RefKernels(a.p, oracle.PRP)
    per = a.ref_iters_per_step
    for _ in range(a.warmup):
        r.iterate(per)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        r.iterate(per)
    dt = time.perf_counter() - t0
    ms_iter = dt / (a.steps * per) * 1e3
    threads = oracle.RefKernels.threads()
    sample = (f"{a.steps} steps x {per} squarings of p={a.p} (n=2^21) through the reference's generic kernel plan, "
              f"{threads} OpenMP threads (OMP_PROC_BIND={os.environ.get('OMP_PROC_BIND')}, "
              f"OMP_PLACES={os.environ.get('OMP_PLACES')})")
    return {
        "impl": "reference", "metric": METRIC, "value": ms_iter, "unit": "ms/iter", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": dt / a.steps * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "iters_per_step": per, "l2": "state and tables resident in host memory"},
        "cpu_baseline": {"value": ms_iter, "unit": "ms/iter", "cores": threads, "kind": "reference", "sample": sample},
        "e2e": {"value": ms_iter, "unit": "ms/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def reference_opencl_gpu(p: int, iters: int) -> dict:
    """The reference program on this GPU (oracle.ref_opencl_run): its own CLI,
    `p prp 1000 -N iters`; ms/iter from the elapsed times it prints at the first
    and the last report (the first 1000 squarings, which include its warm-up,
    are left out)."""
    import re

    import oracle
    rc, out = oracle.ref_opencl_run([str(p), "prp", "1000", "-N", str(iters)], timeout=600)
    pts = [(int(a), float(b)) for a, b in re.findall(r"iter (\d+)/\d+ .*?elapsed ([0-9.]+) s", out)]
    pts = [x for x in pts if x[0] >= 1000]
    if rc != 0 or len(pts) < 2:
        return {"value": None, "sample": f"unavailable: exit {rc}: {out.strip().splitlines()[-1] if out.strip() else ''}"}
    (i0, t0), (i1, t1) = pts[0], pts[-1]
    dev = re.search(r"device=\d+ \(([^)]*)\)", out)
    return {"value": (t1 - t0) / (i1 - i0) * 1e3, "unit": "ms/iter", "kind": "reference",
            "device": dev.group(1) if dev else None,
            "sample": f"mersenne2_gpu.cpp's own OpenCL path on this GPU, squarings {i0}..{i1} of p={p} "
                      f"(its progress lines, one clFinish per 1000)"}


# ---------------------------------------------------------------- n = 2^22
def run_n22(a, stream) -> dict:
    """Config 3's second exponent: the seeded prime in [73400329, 142606333]
    (transform n = 2^22), ms/iter device-timed like the headline (L2 flushed
    between steps), res64 checked against GMP at the golden checkpoints."""
    from mersenne2gpu_gb300.workloads import large_n22_exponent
    return run_one(large_n22_exponent(), 0, a.n22_iters, a.n22_steps, 2, stream)


def run_gf61_only(a, stream) -> dict:
    """The headline exponent in the GF(P61^2)-only layout (the GF61 prototype's
    size rule: n = 2^22 for p = 57885161), timed and checked like n22: the
    same residues as the dual-field transform, with twice the digits."""
    return run_one(a.p, 1, 1000, 2, 1, stream)


def run_one(p, fields, ips, steps, warm, stream) -> dict:
    import torch

    import mersenne2gpu_gb300 as m2
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=stream.device)
    want = {int(k): v for k, v in ((_load_json(GOLDEN_LARGE) or {}).get(str(p), {}).get("prp", {})).items()}
    with m2.Engine(p, m2.MODE_PRP, device=stream.device.index or 0, stream=stream.cuda_stream, fields=fields) as eng:
        info = eng.info()
        for _ in range(warm):
            flush.zero_()
            eng.iterate(ips)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            evs[i][0].record(stream)
            eng.iterate(ips)
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        ms = sum(s.elapsed_time(e) for s, e in evs) / (steps * ips)
        done = (warm + steps) * ips
        parity = None
        if done in want:
            parity = "ok" if f"{eng.res64():016x}" == want[done] else "MISMATCH"
        stages = eng.profile(20)
    return {"p": p, "n": info.n, "fields": "gf61" if fields else "dual", "ms_per_iter": ms, "iters": steps * ips,
            "warmup_iters": warm * ips,
            "plan": {"rows": info.rows, "row_len": info.row_len, "cols_per_cta": info.cols_per_cta,
                     "fused_cols": info.fused_cols},
            f"res64@{done}": parity,
            "stages": [{k: st[k] for k in ("name", "ms_per_launch", "launches")} for st in stages]}


# ---------------------------------------------------------------- error check
def run_gec(a, stream) -> dict:
    """Cost of the Gerbicz error check on the headline exponent: B squarings
    plain, B squarings with the check product updated at their end, and one
    verification (B squarings of the product plus one product), wall-clocked
    on the host after a synchronize; the overhead is amortised over checks
    every B^2 squarings.  The residue at the end is checked against GMP."""
    import time

    import mersenne2gpu_gb300 as m2
    B, blocks = a.gec_block, 4
    want = {int(k): v for k, v in ((_load_json(GOLDEN_LARGE) or {}).get(str(a.p), {}).get("prp", {})).items()}
    with m2.Engine(a.p, m2.MODE_PRP, device=stream.device.index or 0, stream=stream.cuda_stream) as eng:
        eng.iterate(B)                 # warm-up (graph capture, tables)
        eng.sync()
        t0 = time.perf_counter()
        eng.iterate(blocks * B)
        eng.sync()
        plain = (time.perf_counter() - t0) / blocks
        with m2.Gec(eng, B) as g:
            g.iterate(B)               # warm-up of the second context
            eng.sync()
            t0 = time.perf_counter()
            g.iterate(blocks * B)
            eng.sync()
            with_products = (time.perf_counter() - t0) / blocks
            t0 = time.perf_counter()
            ok = g.check()
            check = time.perf_counter() - t0
            st = g.stats()
        done = (2 + 2 * blocks) * B
        parity = None
        if done in want:
            parity = "ok" if f"{eng.res64():016x}" == want[done] else "MISMATCH"
    overhead = (with_products - plain) / plain + check / (B * plain)
    return {"p": a.p, "block": B, "ms_per_block_plain": plain * 1e3, "ms_per_block_with_product": with_products * 1e3,
            "ms_per_check": check * 1e3, "check_passed": ok, "updates": st["updates"],
            "overhead_frac_checks_every_B2": overhead, f"res64@{done}": parity}


# ---------------------------------------------------------------- batched
def run_batched(count: int, plain_sample: int, mul_peak: float | None = None) -> dict:
    import mersenne2gpu_gb300 as m2
    from mersenne2gpu_gb300.workloads import batch_exponents
    ps = batch_exponents(count)
    br = m2.batch_run(ps)
    tests_per_s = count / br.seconds if br.seconds > 0 else None
    # integer-multiply roofline of the batch: sum over tests of p squarings x W(h)
    wide = sum(p * wide_mul_count(m2.layout(p)[1] // 2) for p in ps)
    roof = None
    if mul_peak and br.seconds > 0:
        roof = {"wide_muls": wide, "peak_products_per_s": mul_peak, "t_mul_s": wide / mul_peak,
                "achieved_products_per_s": wide / br.seconds, "frac": (wide / mul_peak) / br.seconds}
    # plain path: one test at a time, a stratified sample over the sorted exponents
    order = sorted(range(count), key=lambda i: ps[i])
    pick = [order[int((k + 0.5) * count / plain_sample)] for k in range(plain_sample)]
    import torch
    tot, same = 0.0, 0
    for i in pick:
        with m2.Engine(ps[i], m2.MODE_PRP) as e:
            e.sync()
            t0 = time.perf_counter()
            e.iterate(ps[i])
            e.sync()
            tot += time.perf_counter() - t0
            same += int(e.res64() == int(br.res64[i]))
    plain_per_test = tot / plain_sample
    plain_tests_per_s = 1.0 / plain_per_test if plain_per_test > 0 else None
    return {
        "config": f"{count} PRP tests, seeded primes in [3, 159739] (n = 8 ... 4096), full runs",
        "tests": count, "seconds": br.seconds, "tests_per_s": tests_per_s,
        "squarings_per_s": br.squarings / br.seconds if br.seconds > 0 else None,
        "plain_tests_per_s": plain_tests_per_s,
        "plain_sample": f"{plain_sample} tests one at a time (stratified by p), mean time extrapolated",
        "speedup_vs_plain": (tests_per_s / plain_tests_per_s) if (tests_per_s and plain_tests_per_s) else None,
        "bit_exact_vs_plain": f"{same}/{plain_sample}", "buckets": br.buckets, "launches": br.launches,
        "primes_found": int(br.is_prime.sum()), "roofline_imad": roof,
        "tuned_per_bucket": {f"n=2^{ln}": {k: (round(v, 1) if isinstance(v, float) else v) for k, v in t.items()}
                             for ln in range(3, 15) if (t := m2.batch_tuning(ln)) is not None},
    }


# ---------------------------------------------------------------- main arm
def run_gb300(a, dist: Dist) -> dict | None:
    import numpy as np
    import torch

    import mersenne2gpu_gb300 as m2
    from mersenne2gpu_gb300 import build as b
    if dist.rank == 0 or dist.world > 1:
        b.build()
    dev = dist.local
    torch.cuda.set_device(dev)
    # One non-default stream carries the L2 flush, the engine's kernels and the
    # timing events (handle 0 would be the legacy stream, which the engine
    # does not run on).
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    eng = m2.Engine(a.p, m2.MODE_PRP, device=dev, stream=stream.cuda_stream)
    info = eng.info()
    ips = a.iters_per_step
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    golden = _load_json(GOLDEN_LARGE) or {}
    want = {int(k): v for k, v in golden.get(str(a.p), {}).get("prp", {}).items()}
    parity = {}

    def check(at: int):
        if at in want:
            got = f"{eng.res64():016x}"
            parity[f"res64@{at}"] = "ok" if got == want[at] else f"MISMATCH {got} != {want[at]}"

    done = 0
    for w in range(a.warmup):
        flush.zero_()
        eng.iterate(ips)
        done += ips
        check(done)
    torch.cuda.synchronize()
    dist.barrier()
    clocks = ClockSampler(dev)
    clocks.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    t0 = time.perf_counter()
    for i in range(a.steps):
        flush.zero_()
        evs[i][0].record(stream)
        eng.iterate(ips)
        evs[i][1].record(stream)
        done += ips
        # a step boundary at a golden checkpoint: the residue is read between
        # the events (outside the device-timed interval of every step)
        check(done)
    torch.cuda.synchronize()
    dist.barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_ms = sum(s.elapsed_time(e) for s, e in evs)
    total_iters = (a.warmup + a.steps) * ips
    dev_ms = dist.max(dev_ms)
    ms_iter_rank = dev_ms / (a.steps * ips)
    value = ms_iter_rank / dist.world

    # e2e: through the C ABI with host buffers in pinned memory (digits in,
    # squarings, canonical digits out; both copies inside the timed region)
    pinned = torch.empty(info.n, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    eng.digits(out=pinned)
    it = eng.info().iteration
    torch.cuda.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for i in range(a.steps):
        eng.set_digits(pinned, it)
        eng.iterate(ips)
        eng.digits(out=pinned)
        it += ips
    dist.barrier()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = e2e_s * 1e3 / (a.steps * ips) / dist.world
    h2d = 8 * info.n
    d2h = 8 * info.n          # canonical digits, carried on the device (m2_get_digits)

    # per-kernel device times for the roofline
    stages = eng.profile(a.profile_iters)
    # dominant kernel: the largest share of the squarings' device time
    dom = max(stages, key=lambda s: s["ms_per_launch"] * s["launches"])
    peaks = _load_json(PEAKS) or {}
    hbm = float(peaks.get("hbm_gbs") or 6800.0)
    peak_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    achieved = dom["bytes_per_launch"] / (dom["ms_per_launch"] * 1e-3) / 1e9
    traffic = (_load_json(TRAFFIC) or {}).get(dom["name"])
    mul_peak = m2.measure_mul_peak(dev)
    h = info.n // 2
    W = wide_mul_count(h)
    B = 48 * h
    t_hbm = B / (hbm * 1e9) * 1e3
    t_mul = W / mul_peak * 1e3
    launches = a.steps * eng.launches_for(ips)   # engine kernels in the timed region
    eng.close()

    if dist.rank != 0:
        return None
    out = {
        "metric": METRIC, "value": value, "unit": "ms/iter", "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": dev_ms / a.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (fixed exponent, state from x0 = 3)",
        "config": {"workload": WORKLOAD, "iters_per_step": ips, "path": "three-pass",
                   "plan": {"rows": info.rows, "row_len": info.row_len, "cols_per_cta": info.cols_per_cta,
                            "carry_span": info.span},
                   "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MB write), state stays L2-resident within a step",
                   "parity_reads": "res64 read between the CUDA-event windows at every step boundary that is a GMP "
                                   "checkpoint; the read's carry kernels are not counted in gpu_launches",
                   "parallelism": "replicas" if dist.world > 1 else "single"},
        "wall_s": wall,
        "gpu_launches": launches,
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": "ms/iter", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic,
                     "bytes_per_launch": dom["bytes_per_launch"], "ms_per_launch": dom["ms_per_launch"],
                     "peak_source": f"{peak_src} hbm_gbs"},
        "roofline_imad": {"wide_muls_per_iter": W, "peak_products_per_s": mul_peak, "t_mul_ms": t_mul,
                          "bytes_per_iter": B, "t_hbm_ms": t_hbm, "roofline_ms": max(t_hbm, t_mul),
                          "frac": max(t_hbm, t_mul) / ms_iter_rank,
                          "achieved_products_per_s": W / (ms_iter_rank * 1e-3)},
        "stages": [{k: s[k] for k in ("name", "ms_per_launch", "launches", "bytes_per_launch")} for s in stages],
        "parity": parity or None,
    }
    if a.cpu_baseline and dist.world == 1:
        try:
            ms, thr, setup = reference_sample(a.p, a.cpu_iters)
            out["cpu_baseline"] = {"value": ms, "unit": "ms/iter", "cores": thr, "kind": "reference",
                                   "sample": f"{a.cpu_iters} squarings of p={a.p} (n=2^21) through the reference's "
                                             f"own kernels on the host cores, {thr} OpenMP threads "
                                             f"(OMP_PROC_BIND={os.environ.get('OMP_PROC_BIND')}, "
                                             f"OMP_PLACES={os.environ.get('OMP_PLACES')}; table setup {setup:.1f} s untimed)"}
            try:
                out["cpu_baseline"]["single_thread"] = {
                    "value": reference_single_thread(a.p, 2), "unit": "ms/iter", "cores": 1, "kind": "reference",
                    "sample": f"2 squarings of p={a.p} through the reference's own kernels on one host thread"}
            except Exception as ex:  # noqa: BLE001
                out["cpu_baseline"]["single_thread"] = {"value": None, "sample": f"unavailable: {ex}"}
        except Exception as ex:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "unit": "ms/iter", "cores": 0, "kind": "reference",
                                   "sample": f"unavailable: {ex}"}
    if a.cpu_baseline and dist.world == 1 and isinstance(out.get("cpu_baseline"), dict):
        try:
            out["cpu_baseline"]["gmp_single_thread"] = gmp_sample(a.p, 3)
        except Exception as ex:  # noqa: BLE001
            out["cpu_baseline"]["gmp_single_thread"] = {"value": None, "sample": f"unavailable: {ex}"}
    if a.ref_opencl and dist.world == 1:
        try:
            out["reference_opencl_gpu"] = reference_opencl_gpu(a.p, 3000)
        except Exception as ex:  # noqa: BLE001
            out["reference_opencl_gpu"] = {"value": None, "sample": f"unavailable: {ex}"}
    if a.n22 and dist.world == 1:
        try:
            out["n22"] = run_n22(a, stream)
        except Exception as ex:  # noqa: BLE001
            out["n22"] = {"error": str(ex)}
    if a.gf61 and dist.world == 1:
        try:
            out["gf61_only"] = run_gf61_only(a, stream)
        except Exception as ex:  # noqa: BLE001
            out["gf61_only"] = {"error": str(ex)}
    if a.gec and dist.world == 1:
        try:
            out["gerbicz"] = run_gec(a, stream)
        except Exception as ex:  # noqa: BLE001
            out["gerbicz"] = {"error": str(ex)}
    if a.batch:
        try:
            out["batched"] = run_batched(a.batch_count, a.plain_sample, mul_peak)
        except Exception as ex:  # noqa: BLE001
            out["batched"] = {"error": str(ex)}
    if a.serve:
        try:
            from mersenne2gpu_gb300.serve import run_serving
            out["serving"] = run_serving(rate_per_s=a.serve_rate, window_s=a.serve_window, device=dev)
        except Exception as ex:  # noqa: BLE001
            out["serving"] = {"error": str(ex)}
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=18)   # 3 + 18 steps of 1000: the state ends at GMP's iteration 21000
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--p", type=int, default=DEFAULT_P)
    ap.add_argument("--iters-per-step", type=int, default=1000)
    ap.add_argument("--ref-iters-per-step", type=int, default=40)
    ap.add_argument("--profile-iters", type=int, default=50)
    ap.add_argument("--cpu-iters", type=int, default=400)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-ref-opencl", dest="ref_opencl", action="store_false")
    ap.add_argument("--no-n22", dest="n22", action="store_false")
    ap.add_argument("--no-gf61", dest="gf61", action="store_false")
    ap.add_argument("--n22-iters", type=int, default=2500)
    ap.add_argument("--n22-steps", type=int, default=6)   # (2 + 6) x 2500: checked at GMP's iteration 20000
    ap.add_argument("--no-gec", dest="gec", action="store_false")
    ap.add_argument("--gec-block", type=int, default=1000)
    ap.add_argument("--no-batch", dest="batch", action="store_false")
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--plain-sample", type=int, default=8)
    ap.add_argument("--no-serve", dest="serve", action="store_false")
    ap.add_argument("--serve-rate", type=float, default=4.0)
    ap.add_argument("--serve-window", type=float, default=20.0)
    a = ap.parse_args()
    if a.warmup < 3:
        a.warmup = 3
    dist = Dist()
    try:
        res = run_reference(a, dist) if a.impl == "reference" else run_gb300(a, dist)
    finally:
        dist.close()
    if res is not None:
        print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
