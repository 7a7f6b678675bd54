"""Generate the golden fixtures of tests/golden/ (committed; the tests only read them).

Sources, cross-checked before anything is written:
  * GMP (gmp_chain.c, built against libgmp.so.10): res64 / full residues;
  * the oracle (oracle/m2_oracle.c) where it finishes in reasonable time;
  * the reference's own kernels (oracle/_ref) where they are built.

The reference ships no golden vectors of its own: results are pinned by the
mathematics (M_9941, M_11213 ... are prime; README.md:55-58) and by GMP.

Usage:
  python tests/golden/make_golden.py --cache DIR [--what small,c1,mid,large,batch] [--jobs N]
DIR keeps the raw gmp_chain outputs so that long runs (p = 57885161, 115640321:
about 0.5-1 s per squaring) are computed once.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SMALL_P = [3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 61, 89, 107, 127, 521, 607, 1279, 2203, 2281, 3217, 4253, 4423,
           9689, 9941, 11213, 19937, 21701, 23209, 44497, 8191, 8209, 10007, 30011]
# p = 57885161: every 1000 squarings up to 30000, so that a bench run of up to 30
# report batches of 1000 ends on a checkpoint whatever its warm-up/timed split
LARGE = {57885161: list(range(1000, 30001, 1000)), 115640321: [1000, 10000, 20000, 21000]}
LARGE_LL = {57885161: [1000], 115640321: [1000]}   # the LL -2 step through the n = 2^21 / 2^22 kernels


def gmp_bin(cache: str) -> str:
    out = os.path.join(cache, "gmp_chain")
    src = os.path.join(HERE, "gmp_chain.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-o", out, src, "-l:libgmp.so.10"], check=True)
    return out


def gmp_run(cache: str, p: int, mode: str, iters: int, spec: str, hexout: bool = False) -> dict[int, tuple[str, str | None]]:
    tag = f"gmp_{p}_{mode}_{iters}_{spec.replace(',', '-')}{'_hex' if hexout else ''}.txt"
    path = os.path.join(cache, tag)
    if not os.path.exists(path):
        cmd = [gmp_bin(cache), str(p), mode, str(iters), spec] + (["--hex"] if hexout else [])
        with open(path + ".tmp", "w") as f:
            subprocess.run(cmd, check=True, stdout=f)
        os.replace(path + ".tmp", path)
    out = {}
    for line in open(path):
        f = line.split()
        if len(f) >= 4 and f[0] == "iter":
            out[int(f[1])] = (f[3], f[5] if len(f) >= 6 else None)
    return out


def total(p: int, mode: str) -> int:
    return {"ll": p - 2, "prp": p, "prp3": p - 1}[mode]


def make_small(cache: str, jobs: int) -> dict:
    import oracle
    res = {}
    tasks = [(p, m) for p in SMALL_P for m in ("ll", "prp", "prp3")]
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = {t: ex.submit(gmp_run, cache, t[0], t[1], total(*t), str(total(*t))) for t in tasks}
    for (p, m), fu in futs.items():
        r = fu.result()[total(p, m)][0]
        o = oracle.Oracle(p, {"ll": 0, "prp": 1, "prp3": 2}[m])
        o.iterate(total(p, m))
        assert f"{o.res64():016x}" == r, (p, m, o.res64(), r)
        want = {"ll": 0, "prp": 9, "prp3": 3}[m] % ((1 << p) - 1)
        res.setdefault(str(p), {})[m] = {"iters": total(p, m), "res64": r, "prime": int(r, 16) == want and
                                         o.verdict()}
    return res


def make_c1(cache: str) -> dict:
    import oracle
    out = {}
    for m in ("prp", "ll"):
        T = total(9941, m)
        g = gmp_run(cache, 9941, m, T, "1000", hexout=True)
        o = oracle.Oracle(9941, {"ll": 0, "prp": 1}[m])
        w = o.widths()
        ref = oracle.RefKernels(9941, {"ll": 0, "prp": 1}[m]) if oracle.ref_available() else None
        done, ck = 0, {}
        for it in sorted(g):
            o.iterate(it - done)
            if ref is not None:
                ref.iterate(it - done)
            done = it
            v = int(g[it][1], 16)
            d = o.digits()
            assert oracle.value_of_digits(d, w) == v, (m, it)
            if ref is not None:
                assert (ref.digits() == d).all(), (m, it, "reference kernels")
            ck[str(it)] = g[it][1]
        out[m] = {"checkpoints_hex": ck, "prime": bool(o.verdict())}
    return out


def make_mid(cache: str, jobs: int) -> dict:
    from mersenne2gpu_gb300.workloads import mid_exponents
    out = {}
    runs = [(132049, m, total(132049, m)) for m in ("prp", "ll")]
    runs += [(p, m, 10000) for p in mid_exponents() for m in ("prp", "ll")]
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = {r: ex.submit(gmp_run, cache, r[0], r[1], r[2], "1000") for r in runs}
    for (p, m, it), fu in futs.items():
        out.setdefault(str(p), {})[m] = {str(k): v[0] for k, v in sorted(fu.result().items())}
    # oracle cross-check of the first checkpoints
    import oracle
    for p in [132049] + mid_exponents()[:4]:
        for m in ("prp", "ll"):
            o = oracle.Oracle(p, {"ll": 0, "prp": 1}[m])
            o.iterate(1000)
            assert f"{o.res64():016x}" == out[str(p)][m]["1000"], (p, m)
    return out


def make_large(cache: str, jobs: int) -> dict:
    out = {}
    runs = [(p, "prp", c) for p, c in LARGE.items()] + [(p, "ll", c) for p, c in LARGE_LL.items()]
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = {(p, m): ex.submit(gmp_run, cache, p, m, max(c), ",".join(map(str, c))) for p, m, c in runs}
    for (p, m), fu in futs.items():
        out.setdefault(str(p), {})[m] = {str(k): v[0] for k, v in sorted(fu.result().items())}
    return out


def make_batch(cache: str, jobs: int, count: int = 4096, cap: int = 2000) -> dict:
    """res64 after min(p, cap) squarings for the seeded batch exponents (PRP)."""
    from mersenne2gpu_gb300.workloads import batch_exponents
    ps = batch_exponents(count)
    uniq = sorted(set(ps))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = {p: ex.submit(gmp_run, cache, p, "prp", min(p, cap), str(min(p, cap))) for p in uniq}
    return {"cap": cap, "count": count, "res64": {str(p): futs[p].result()[min(p, cap)][0] for p in uniq}}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cache", required=True)
    ap.add_argument("--what", default="small,c1,mid,large,batch")
    ap.add_argument("--jobs", type=int, default=max(1, (os.cpu_count() or 2) - 1))
    a = ap.parse_args()
    os.makedirs(a.cache, exist_ok=True)
    gmp_bin(a.cache)   # build once, before any worker thread runs it
    what = set(a.what.split(","))
    import oracle
    oracle.build()
    meta = {"generator": "tests/golden/make_golden.py", "gmp": "libgmp.so.10 via gmp_chain.c"}
    if "small" in what:
        json.dump({"meta": meta, "tests": make_small(a.cache, a.jobs)}, open(os.path.join(HERE, "small.json"), "w"), indent=1)
    if "c1" in what:
        json.dump({"meta": meta, "p": 9941, "modes": make_c1(a.cache)}, open(os.path.join(HERE, "config1_9941.json"), "w"), indent=1)
    if "mid" in what:
        json.dump(make_mid(a.cache, a.jobs), open(os.path.join(HERE, "mid.json"), "w"), indent=1)
    if "large" in what:
        json.dump(make_large(a.cache, a.jobs), open(os.path.join(HERE, "large.json"), "w"), indent=1)
    if "batch" in what:
        json.dump(make_batch(a.cache, a.jobs), open(os.path.join(HERE, "batch.json"), "w"), indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
