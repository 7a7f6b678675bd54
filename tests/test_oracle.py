"""The CPU oracle pinned against the golden vectors (GMP) and the reference's own kernels."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
MODES = {"ll": 0, "prp": 1, "prp3": 2}


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_small_golden(oracle_mod):
    """Full runs of small exponents (primes and composites), all three modes."""
    g = _load("small.json")["tests"]
    for p, modes in g.items():
        if int(p) > 12000:
            continue   # the longer full runs are checked on the GPU (tests/test_gpu_golden.py)
        for m, rec in modes.items():
            o = oracle_mod.Oracle(int(p), MODES[m])
            o.iterate(rec["iters"])
            assert f"{o.res64():016x}" == rec["res64"], (p, m)
            assert o.verdict() == rec["prime"], (p, m)


def test_known_primes_and_composites(oracle_mod):
    """M_p prime for p in the reference README's examples that finish quickly (README.md:55-56)."""
    g = _load("small.json")["tests"]
    for p in ("3", "5", "7", "13", "17", "19", "31", "61", "89", "107", "127", "521", "607", "1279", "9941", "11213"):
        assert g[p]["ll"]["prime"] and g[p]["prp"]["prime"], p
    for p in ("11", "23", "29", "8191", "8209", "10007", "30011"):
        assert not g[p]["ll"]["prime"] and not g[p]["prp"]["prime"], p


def test_config1_state_every_1000(oracle_mod):
    """p = 9941, n = 256: the full residue every 1000 iterations equals GMP's."""
    g = _load("config1_9941.json")
    for m in ("prp", "ll"):
        o = oracle_mod.Oracle(9941, MODES[m])
        w = o.widths()
        done = 0
        for it, hx in sorted(((int(k), v) for k, v in g["modes"][m]["checkpoints_hex"].items())):
            o.iterate(it - done)
            done = it
            assert oracle_mod.value_of_digits(o.digits(), w) == int(hx, 16), (m, it)
        assert o.verdict() == g["modes"][m]["prime"]


@pytest.mark.parametrize("p", [132049, 237487])
def test_mid_first_checkpoints(oracle_mod, p):
    g = _load("mid.json")[str(p)]
    for m in ("prp", "ll"):
        o = oracle_mod.Oracle(p, MODES[m])
        o.iterate(1000)
        assert f"{o.res64():016x}" == g[m]["1000"], (p, m)


def test_batch_golden_subset(oracle_mod):
    g = _load("batch.json")
    ps = sorted(int(p) for p in g["res64"])[:40]
    for p in ps:
        o = oracle_mod.Oracle(p, 1)
        o.iterate(min(p, g["cap"]))
        assert f"{o.res64():016x}" == g["res64"][str(p)], p


def test_python_chain_agrees(oracle_mod):
    for p in (61, 89, 127, 521):
        for m in (0, 1, 2):
            o = oracle_mod.Oracle(p, m)
            o.iterate(100)
            _, w = o.n, o.widths()
            assert oracle_mod.value_of_digits(o.digits(), w) == oracle_mod.python_chain(p, m, 100), (p, m)


def test_reference_kernels_match_oracle(oracle_mod):
    """The reference's own OpenCL kernels (compiled for the CPU) give the oracle's digits."""
    if not oracle_mod.ref_available():
        pytest.skip("reference kernel sources not extracted on this machine")
    for p in (3, 7, 31, 127, 1279, 9941, 21701):
        for m in (0, 1):
            for cp in (1, 64):
                o, r = oracle_mod.Oracle(p, m), oracle_mod.RefKernels(p, m, cp)
                k = min(p, 150)
                o.iterate(k)
                r.iterate(k)
                assert np.array_equal(o.digits(), r.digits()), (p, m, cp)


def test_oracle_detects_planted_fault(oracle_mod):
    """A bit flipped in a host copy of the state is caught by the comparison."""
    o1, o2 = oracle_mod.Oracle(9941, 1), oracle_mod.Oracle(9941, 1)
    o1.iterate(10)
    o2.iterate(10)
    d = o2.digits()
    d[17] ^= np.uint64(1 << 5)
    o2.set_digits(d, 10)
    o1.iterate(5)
    o2.iterate(5)
    assert not np.array_equal(o1.digits(), o2.digits())
