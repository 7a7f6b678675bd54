"""Gerbicz error check of PRP chains (m2_gec_*): every check of a correct
chain passes, and a wrong state is caught and rolled back.

The wrong state is made on the host: the test reads the digits, flips one bit
and writes them back through m2_set_digits (no GPU fault).  Results after a
rollback must equal the GMP golden residues.
"""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _golden(name):
    with open(os.path.join(HERE, "golden", name)) as f:
        return json.load(f)


def _flip(e):
    d = e.digits()
    d[0] ^= np.uint64(1)
    e.set_digits(d, e.info().iteration)


def _run_checked(g, upto, every, flip_at=None, chunk=37):
    """Advance to iteration `upto` in chunks, checking every `every` squarings;
    returns the list of (iteration, passed) of the checks."""
    e = g.engine
    log, flipped, last = [], False, e.info().iteration
    while e.info().iteration < upto:
        it = e.info().iteration
        g.iterate(min(chunk, upto - it))
        it = e.info().iteration
        if flip_at is not None and not flipped and it >= flip_at:
            _flip(e)
            flipped = True
        if it - last >= every or it == upto:
            ok = g.check()
            log.append((it, ok))
            last = g.verified_iter
            assert e.info().iteration == g.verified_iter
    return log


def test_gec_full_chain_one_cta(m2):
    """M_9941 (n = 256, one-CTA path): a full PRP with B = 10, checked every
    100 squarings; every check passes and the verdict is prime."""
    with m2.Engine(9941, "prp") as e, m2.Gec(e, 10) as g:
        log = _run_checked(g, 9941, 100)
        assert all(ok for _, ok in log) and len(log) >= 80
        assert e.verdict() and e.res64() == 9
        st = g.stats()
        # products restart with every verified state: 11 per 111 squarings
        assert st["failures"] == 0 and st["updates"] >= 880 and st["verified_iter"] == 9941
        assert st["checks"] == len(log)


def test_gec_catches_flip_one_cta(m2):
    with m2.Engine(9941, "prp") as e, m2.Gec(e, 10) as g:
        log = _run_checked(g, 9941, 100, flip_at=250)
        fails = [it for it, ok in log if not ok]
        assert len(fails) == 1 and g.stats()["failures"] == 1
        assert e.verdict() and e.res64() == 9


def test_gec_catches_flip_three_pass_n2_21(m2):
    """p = 57885161 (n = 2^21, three-pass path with the fused column pass):
    B = 100, checks every 500 squarings, one bit flipped at 700; the check at
    1000 fails, the chain goes back to 500, and the residue at 1000 equals GMP's."""
    want = _golden("large.json")["57885161"]["prp"]["1000"]
    with m2.Engine(57885161, "prp") as e, m2.Gec(e, 100) as g:
        assert e.info().path == m2.PATH_LARGE
        log = _run_checked(g, 1000, 500, flip_at=700, chunk=100)
        assert [ok for _, ok in log] == [True, False, True], log
        assert log[1][0] == 1000 and g.verified_iter == 1000
        assert f"{e.res64():016x}" == want


def test_gec_catches_flip_n2_22(m2):
    """p = 115640321 (n = 2^22: the fused column pass with groups taken by
    arrival ticket): B = 100, checks every 300 squarings, one bit flipped at 350."""
    want = _golden("large.json")["115640321"]["prp"]["1000"]
    with m2.Engine(115640321, "prp") as e, m2.Gec(e, 100) as g:
        assert e.info().path == m2.PATH_LARGE and e.info().n == 1 << 22
        log = _run_checked(g, 1000, 300, flip_at=350, chunk=50)
        assert [ok for _, ok in log] == [True, False, True, True, True], log
        assert f"{e.res64():016x}" == want


def test_gec_tail_only_and_mid_size(m2):
    """Checks inside the first block (nothing but repeated squarings to
    compare) on p = 132049 (n = 4096, three-pass path), against GMP."""
    want = _golden("mid.json")["132049"]["prp"]
    with m2.Engine(132049, "prp") as e, m2.Gec(e, 1000) as g:
        g.iterate(250)
        assert g.check() and g.verified_iter == 250
        g.iterate(250)
        _flip(e)
        assert not g.check() and g.verified_iter == 250 and e.info().iteration == 250
        g.iterate(750)
        assert g.check() and g.verified_iter == 1000
        assert f"{e.res64():016x}" == want["1000"]
        d, it = g.verified()
        assert it == 1000 and np.array_equal(d, e.digits())


def test_gec_gf61_fields(m2):
    """GF(P61^2)-only transform: same residues as the two-field engine."""
    with m2.Engine(44497, "prp", fields=m2.FIELDS_GF61) as e, m2.Gec(e, 16) as g:
        log = _run_checked(g, 2000, 256, flip_at=1000)
        assert sum(not ok for _, ok in log) == 1
        r = e.res64()
    with m2.Engine(44497, "prp") as ref:
        ref.iterate(2000)
        assert r == ref.res64()


def test_gec_refuses_ll_prp3_and_zero_block(m2):
    for mode in ("ll", "prp3"):   # no x_(k+B) = x_k^(2^B) relation
        with m2.Engine(9941, mode) as e:
            with pytest.raises(m2.M2Error) as ei:
                m2.Gec(e, 10)
            assert ei.value.code == -6
    with m2.Engine(9941, "prp") as e:
        with pytest.raises(m2.M2Error) as ei:
            m2.Gec(e, 0)
        assert ei.value.code == -1


def test_cli_gerbicz_catches_flip(m2, tmp_path):
    exe = os.path.join(ROOT, "mersenne2gpu_gb300", "mersenne2")
    ck = str(tmp_path / "state.m2")
    r = subprocess.run([exe, "9941", "prp", "500", "--gerbicz", "20", "--debug-gec-corrupt", "700",
                        "--checkpoint", ck], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-500:]
    assert "debug: one bit of the state flipped at iter 1000" in r.stdout, r.stdout
    assert "gerbicz check failed at iter 1000, back to iter 500" in r.stdout, r.stdout
    assert "gerbicz check passed at iter 9941" in r.stdout, r.stdout
    assert "2^9941 - 1 is a probable prime" in r.stdout
    assert "failures=1" in r.stdout and "res64=0000000000000009" in r.stdout
    r = subprocess.run([exe, "9941", "ll", "--gerbicz", "20"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "prp only" in r.stderr
