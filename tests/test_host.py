"""Host-side logic and the C ABI surface, no GPU needed (no compute calls)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The reference's exponent -> n table (README.md:69-102); rows 1-2 of the README
# (3-173 -> 4, 179-349 -> 8) disagree with its own code, which gives n = 8 for
# every exponent up to 349 (mersenne2_gpu.cpp:286-293): the code is authoritative.
README_TABLE = [
    (3, 173, 8), (179, 349, 8), (353, 683, 16), (691, 1373, 32), (1381, 2687, 64), (2689, 5351, 128),
    (5381, 10487, 256), (10499, 20983, 512), (21001, 40949, 1024), (40961, 81919, 2048), (81929, 159739, 4096),
    (159763, 319483, 8192), (319489, 622577, 16384), (622603, 1245169, 32768), (1245187, 2424827, 65536),
    (2424833, 4849651, 131072), (4849687, 9437179, 262144), (9437189, 18874367, 524288),
    (18874379, 36700159, 1048576), (36700201, 73400311, 2097152), (73400329, 142606333, 4194304),
    (142606357, 285212659, 8388608), (285212677, 553648103, 16777216), (553648171, 1107296251, 33554432),
    (1107296257, 2147483647, 67108864),
]


def test_transform_table(m2, oracle_mod):
    for lo, hi, n in README_TABLE:
        for p in (lo, hi):
            ln, nn, _ = m2.layout(p) if p < 40_000_000 else (None, None, None)
            want = n.bit_length() - 1
            assert oracle_mod.transformsize(p) == want, p
            if ln is not None:
                assert (ln, nn) == (want, n), p


@pytest.mark.parametrize("p", [3, 5, 7, 31, 127, 9941, 132049, 216091, 1398269, 9437179])
def test_layout_matches_oracle(m2, oracle_mod, p):
    ln, n, w = m2.layout(p)
    o = oracle_mod.Oracle(p, 1)
    assert (ln, n) == (o.ln, o.n)
    assert np.array_equal(w, o.widths())
    assert int(w.astype(np.int64).sum()) == p
    q = p >> ln
    assert set(np.unique(w).tolist()) <= {q, q + 1}


def _header_symbols():
    src = open(os.path.join(ROOT, "include", "m2gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(m2_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(m2):
    syms = _header_symbols()
    assert "m2_create" in syms and "m2_square_noalloc" in syms
    lib = m2._lib()
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(m2.EXPORTS) == syms


def test_strerror_codes(m2):
    lib = m2._lib()
    for code in range(0, -7, -1):
        assert lib.m2_strerror(code)
    assert lib.m2_strerror(-1) == b"invalid argument"


def test_invalid_arguments_rejected_without_device(m2):
    import ctypes
    lib = m2._lib()
    h = ctypes.c_void_p()
    assert lib.m2_create(ctypes.byref(h), 2, 1, None) == -1     # p < 3
    assert lib.m2_create(ctypes.byref(h), 9941, 7, None) == -1  # bad mode
    assert lib.m2_iterate(None, 1) == -1
    assert lib.m2_layout(1, None, None, None) == -1


def _cli():
    return os.path.join(ROOT, "mersenne2gpu_gb300", "mersenne2")


def test_cli_usage_and_argument_errors(m2):
    exe = _cli()
    assert os.path.exists(exe)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage:" in r.stderr and "[ll|prp] [report_every]" in r.stderr
    r = subprocess.run([exe, "9941", "prp", "100", "junk"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown argument: junk" in r.stderr
    r = subprocess.run([exe, "9941", "-d"], capture_output=True, text=True)
    assert r.returncode == 1 and "Missing device id after -d" in r.stderr
    r = subprocess.run([exe, "9941", "-B"], capture_output=True, text=True)
    assert r.returncode == 1 and "Missing carry_pairs after -B" in r.stderr


def test_cli_first_line_without_gpu(m2):
    """The transform line comes before any device work (mersenne2_gpu.cpp:3733)."""
    from conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present; covered by the GPU CLI test")
    r = subprocess.run([_cli(), "57885161", "prp"], capture_output=True, text=True)
    assert r.stdout.splitlines()[0] == "p=57885161, ln=21, transform=1048576 (n=2097152)"
    assert r.returncode == 1


def _gf61_log2(p):
    """The GF61 prototype's size rule (gf61_ntt_prp_opencl_inplace_nobitrev_fused.cpp:124-132)."""
    ln = 2
    while True:
        ln += 1
        if ln + 2 * ((p >> ln) + 1) < 61:
            return ln


@pytest.mark.parametrize("p", [3, 7, 31, 89, 127, 521, 9941, 44497, 132049, 216091, 376831])
def test_gf61_layout_follows_the_prototype_rule(m2, p):
    ln, n, w = m2.layout(p, m2.FIELDS_GF61)
    assert ln == _gf61_log2(p) and n == 1 << ln
    assert int(w.sum()) == p and set(np.unique(w)) <= {p >> ln, (p >> ln) + 1}


def test_cli_gf61_first_line_without_gpu(m2):
    from conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present; covered by the GPU tests")
    r = subprocess.run([_cli(), "216091", "prp", "--gf61"], capture_output=True, text=True)
    assert r.stdout.splitlines()[0] == "p=216091, ln=14, transform=8192 (n=16384)"
    assert r.returncode == 1


@pytest.mark.parametrize("p", [3, 7, 31, 127, 9941, 132049, 2976221, 18874367, 57885161, 115640321])
def test_carry_width_rule_matches_layout(m2, p):
    """The kernels' carry loops take digit j's width as q + [((p j - 1) mod n)
    + (p mod n) >= n] (q + [p mod n != 0] for j = 0), the remainder formed in
    32-bit arithmetic; it must equal the layout's ceil(p (j+1) / n) -
    ceil(p j / n) for every digit, in both field layouts."""
    for fields in (m2.FIELDS_DUAL, m2.FIELDS_GF61):
        ln, n, widths = m2.layout(p, fields)
        nm, pm, q = n - 1, p & (n - 1), p >> ln
        j = np.arange(n, dtype=np.uint64)
        r = ((j * np.uint64(pm) - np.uint64(1)) & np.uint64(0xFFFFFFFF)) & np.uint64(nm)
        w = np.uint64(q) + ((r + np.uint64(pm)) >> np.uint64(ln))
        w[0] = q + (1 if pm else 0)
        assert np.array_equal(w.astype(np.uint8), widths), (p, fields)


def test_digit_to_p31_rule():
    """A signed digit or pending carry d (|d| < 2^62) reaches GF(P31) as
    (d + P31 2^32) mod P31 through one unsigned 64-bit reduction."""
    P31 = (1 << 31) - 1

    def red31(x):
        r = (x & P31) + (x >> 31)
        s = ((r & P31) + (r >> 31)) & 0xFFFFFFFF
        return min(s, (s - P31) & 0xFFFFFFFF)

    rng = np.random.default_rng(3)
    ds = [0, 1, -1, P31, -P31, (1 << 62) - 1, -(1 << 62) + 1] + [int(x) for x in rng.integers(-(1 << 62), 1 << 62, 2000)]
    for d in ds:
        got = red31((d + (P31 << 32)) & ((1 << 64) - 1))
        assert 0 <= got <= P31 and got % P31 == d % P31, d
