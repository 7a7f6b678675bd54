"""The CUDA engine against the committed golden vectors (GMP), configs 1-4.

config 1: p = 9941 (n = 256), PRP and LL, full residue every 1000 iterations.
config 2: p = 132049 (n = 4096) full runs, res64 every 1000; 20 seeded primes in
          [159763, 319483] (n = 8192), 10000 iterations, res64 every 1000.
config 3: p = 57885161 (n = 2^21) and a seeded prime in [73400329, 142606333]
          (n = 2^22): PRP res64 at the golden checkpoints (1000 / 10000 / 20000 /
          21000) and LL res64 at 1000.
config 4: the 4096 seeded batch exponents (n = 8 ... 4096) through the batched
          engine, res64 after min(p, 2000) squarings, and batched == plain.
"""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
MODES = {"ll": 0, "prp": 1, "prp3": 2}


def _load(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def test_small_golden_full_runs(m2):
    g = _load("small.json")["tests"]
    for p, modes in g.items():
        for m, rec in modes.items():
            with m2.Engine(int(p), MODES[m]) as e:
                e.iterate(rec["iters"])
                assert f"{e.res64():016x}" == rec["res64"], (p, m)
                assert e.verdict() == rec["prime"], (p, m)


def test_config1_full_state_every_1000(m2, oracle_mod):
    g = _load("config1_9941.json")
    _, _, w = m2.layout(9941)
    for m in ("prp", "ll"):
        with m2.Engine(9941, MODES[m]) as e:
            done = 0
            for it, hx in sorted(((int(k), v) for k, v in g["modes"][m]["checkpoints_hex"].items())):
                e.iterate(it - done)
                done = it
                assert np.array_equal(e.digits(), oracle_mod.digits_of_value(int(hx, 16), w)), (m, it)
            assert e.verdict() == g["modes"][m]["prime"]


@pytest.mark.parametrize("mode", ["prp", "ll"])
def test_config2_132049_full_run(m2, mode):
    g = _load("mid.json")["132049"][mode]
    with m2.Engine(132049, MODES[mode]) as e:
        done = 0
        for it, r in sorted(((int(k), v) for k, v in g.items())):
            e.iterate(it - done)
            done = it
            assert f"{e.res64():016x}" == r, (mode, it)
        assert e.verdict()   # M_132049 is prime


def test_config2_mid_exponents(m2):
    from mersenne2gpu_gb300.workloads import mid_exponents
    g = _load("mid.json")
    for p in mid_exponents():
        for mode in ("prp", "ll"):
            with m2.Engine(p, MODES[mode]) as e:
                done = 0
                for it, r in sorted(((int(k), v) for k, v in g[str(p)][mode].items())):
                    e.iterate(it - done)
                    done = it
                    assert f"{e.res64():016x}" == r, (p, mode, it)


def test_config3_large_checkpoints(m2):
    g = _load("large.json")
    for p, rec in g.items():
        for mode, cp in rec.items():
            with m2.Engine(int(p), MODES[mode]) as e:
                done = 0
                for it in sorted(int(k) for k in cp):
                    e.iterate(it - done)
                    done = it
                    assert f"{e.res64():016x}" == cp[str(it)], (p, mode, it)


def test_config4_batched_golden_and_plain(m2):
    from mersenne2gpu_gb300.workloads import batch_exponents
    g = _load("batch.json")
    ps = batch_exponents(g["count"])
    iters = [min(p, g["cap"]) for p in ps]
    br = m2.batch_run(ps, iters=iters)
    for i, p in enumerate(ps):
        assert f"{int(br.res64[i]):016x}" == g["res64"][str(p)], p
    # every bucket was autotuned over threads per transform (32 ... 256), carry
    # blocks (threads, threads/2, threads/4) and a fused or separate middle,
    # and the choice is never slower than the untuned default it also timed
    for ln in sorted({m2.layout(p)[0] for p in ps}):
        t = m2.batch_tuned(ln)
        assert t is not None and t[0] in (32, 64, 128, 256) and t[1] > 0, (ln, t)
        full_t = m2.batch_tuning(ln)
        assert full_t is not None and full_t["threads"] == t[0], (ln, full_t)
        assert full_t["fused_middle"] in (0, 1) and full_t["carry_blocks"] >= 0, (ln, full_t)
        if full_t["carry_blocks"]:
            assert full_t["carry_blocks"] <= full_t["threads"], (ln, full_t)
            assert full_t["carry_pairs"] * 2 * full_t["carry_blocks"] == 1 << ln, (ln, full_t)
        assert full_t["ns_per_test_squaring"] <= full_t["ns_default"], (ln, full_t)
    # full runs: batched == plain on a spread of exponents (each bucket)
    pick = sorted(set(ps))[:: max(1, len(set(ps)) // 24)]
    full = m2.batch_run(pick)
    for i, p in enumerate(pick):
        with m2.Engine(p, 1) as e:
            e.iterate(p)
            assert e.res64() == int(full.res64[i]), p
            assert e.verdict() == bool(full.is_prime[i]), p


def test_cli_prime_and_composite(m2):
    exe = os.path.join(ROOT, "mersenne2gpu_gb300", "mersenne2")
    r = subprocess.run([exe, "9941", "prp", "-d", "0"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "p=9941, ln=8, transform=128 (n=256)"
    assert lines[1].startswith("device=0 (")
    assert lines[2].startswith("carry_blocks=")
    assert lines[3].startswith("iter 0/9941 (0.0%), elapsed")
    assert any(ln.startswith("iter 9941/9941 (100.0%)") for ln in lines)
    assert "2^9941 - 1 is a probable prime, elapsed" in r.stdout
    assert lines[-1] == "res64=0000000000000009"
    r = subprocess.run([exe, "9949", "ll", "500", "--res64"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "2^9949 - 1 is composite" in r.stdout
    assert ", res64 " in r.stdout
    r = subprocess.run([exe, "11213", "ll", "-N", "3000"], capture_output=True, text=True, timeout=120)
    assert "benchmark_iters=3000" in r.stdout and "iter 3000/3000" in r.stdout


def test_cli_checkpoint_resume(m2, tmp_path):
    exe = os.path.join(ROOT, "mersenne2gpu_gb300", "mersenne2")
    ck = str(tmp_path / "state.m2")
    r = subprocess.run([exe, "21701", "ll", "1000", "-N", "5000", "--checkpoint", ck], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and os.path.exists(ck)
    r2 = subprocess.run([exe, "21701", "ll", "1000", "--resume", ck, "--res64"], capture_output=True, text=True,
                        timeout=300)
    assert r2.returncode == 0 and "resumed at iter 5000" in r2.stdout
    assert "2^21701 - 1 is prime" in r2.stdout     # M_21701 is a Mersenne prime
    # a corrupted state file is refused
    with open(ck, "r+b") as f:
        f.seek(100)
        f.write(b"\xff\xff")
    r3 = subprocess.run([exe, "21701", "ll", "--resume", ck], capture_output=True, text=True, timeout=60)
    assert r3.returncode == 1 and "checksum mismatch" in r3.stderr


def test_cli_sigint_stops_cleanly_and_resumes(m2, tmp_path):
    """SIGINT (host-side fault injection, no GPU fault): the run stops at the
    next report point with its checkpoint written and exit status 130; resuming
    from the checkpoint reaches the same residue as an uninterrupted run."""
    import signal
    import subprocess
    import time
    cli = os.path.join(os.path.dirname(m2.__file__), "mersenne2")
    ck = str(tmp_path / "state.m2")
    args = [cli, "2976221", "prp", "4000", "-N", "400000", "--checkpoint", ck]
    pr = subprocess.Popen(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    t0 = time.time()
    while not os.path.exists(ck) and time.time() - t0 < 60:
        time.sleep(0.05)
    time.sleep(1.0)
    pr.send_signal(signal.SIGINT)
    out, err = pr.communicate(timeout=120)
    assert pr.returncode == 130, (pr.returncode, out[-500:], err[-500:])
    assert "interrupted at iter" in out
    stopped = int(out.split("interrupted at iter ")[1].split(",")[0])
    assert 0 < stopped < 400000
    r2 = subprocess.run([cli, "2976221", "prp", "100000", "-N", "400000", "--resume", ck],
                        capture_output=True, text=True, timeout=300)
    assert r2.returncode == 0, r2.stderr[-500:]
    assert f"resumed at iter {stopped}" in r2.stdout
    r3 = subprocess.run([cli, "2976221", "prp", "100000", "-N", "400000"], capture_output=True, text=True, timeout=300)
    assert r3.returncode == 0
    res = [ln for ln in r2.stdout.splitlines() if ln.startswith("res64=")]
    assert res and res == [ln for ln in r3.stdout.splitlines() if ln.startswith("res64=")]
