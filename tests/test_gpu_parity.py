"""Parity of the CUDA engine against the CPU oracle, through the C ABI.

Bit-exact: the canonical digit vector (the reference's state after its carry,
mersenne2_gpu.cpp:2116) must equal the oracle's at every compared iteration.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TINY = [3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 89, 107, 127]


def _cmp(got, want, what):
    if not np.array_equal(got, want):
        bad = np.nonzero(got != want)[0]
        raise AssertionError(f"{what}: {len(bad)} digits differ, first at {bad[0]}: {got[bad[0]]} != {want[bad[0]]}")


@pytest.mark.parametrize("p", TINY)
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_tiny_exponents_full_run(m2, oracle_mod, p, mode):
    """Tiny p (zero-width digits for p < 8): full runs against exact integers,
    with the one-CTA kernel's middle fused for every other exponent."""
    with m2.Engine(p, mode, fused_middle=TINY.index(p) % 2) as e:
        iters = m2.total_iterations(p, mode)
        e.iterate(iters)
        want = oracle_mod.python_chain(p, mode, iters) % ((1 << p) - 1)
        assert e.res64() == want & ((1 << 64) - 1)
        _, _, w = m2.layout(p)
        _cmp(e.digits(), oracle_mod.digits_of_value(want, w), f"p={p} mode={mode}")
        assert e.verdict() == (want == {0: 0, 1: 9 % ((1 << p) - 1), 2: 3 % ((1 << p) - 1)}[mode])


@pytest.mark.parametrize("mode", [0, 1])
def test_9941_state_every_1000(m2, oracle_mod, mode):
    """Config 1: p = 9941 (n = 256), full run, full state every 1000 iterations."""
    p = 9941
    o = oracle_mod.Oracle(p, mode)
    total = m2.total_iterations(p, mode)
    with m2.Engine(p, mode) as e:
        done = 0
        while done < total:
            k = min(1000, total - done)
            e.iterate(k)
            o.iterate(k)
            done += k
            _cmp(e.digits(), o.digits(), f"p=9941 mode={mode} iter={done}")
        assert e.verdict()   # M_9941 is prime


@pytest.mark.parametrize("p", [521, 1279, 2203, 4423, 9689, 21701, 44497, 86243, 132049, 216091])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("fused", [0, 1])
def test_small_path_vs_oracle(m2, oracle_mod, p, mode, fused):
    """The one-CTA kernel with the transform's middle (last forward level, centre
    square, first inverse level) as separate passes or fused into one pass."""
    iters = 200 if p < 100000 else 60
    with m2.Engine(p, mode, path=m2.PATH_SMALL, fused_middle=fused) as e:
        e.iterate(iters)
        got = e.digits()
    o = oracle_mod.Oracle(p, mode)
    o.iterate(iters)
    _cmp(got, o.digits(), f"small p={p} mode={mode}")


@pytest.mark.parametrize("p", [4423, 9941, 44497, 132049, 216091, 756839, 1398269, 2976221])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_large_path_vs_oracle(m2, oracle_mod, p, mode):
    iters = 40 if p < 1000000 else 6
    with m2.Engine(p, mode, path=m2.PATH_LARGE) as e:
        e.iterate(iters)
        got = e.digits()
    o = oracle_mod.Oracle(p, mode)
    o.iterate(iters)
    _cmp(got, o.digits(), f"large p={p} mode={mode}")


@pytest.mark.parametrize("p", [18874367, 36700159, 57885161, 115640321])   # row pass of 1024 / 2048, 1024-row columns
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_large_path_long_rows_vs_oracle(m2, oracle_mod, p, mode):
    iters = 2
    with m2.Engine(p, mode, path=m2.PATH_LARGE) as e:
        info = e.info()
        assert info.row_len in (1024, 2048)
        e.iterate(iters)
        got = e.digits()
    o = oracle_mod.Oracle(p, mode)
    o.iterate(iters)
    _cmp(got, o.digits(), f"large p={p} mode={mode}")


@pytest.mark.parametrize("p", [2976221, 9437179, 18874367, 36700159])   # R = 256 rows: B = 256, 512, 1024, 2048
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_large_path_256_rows_vs_oracle(m2, oracle_mod, p, mode):
    """R = 256 rows: the generic column kernels (B = 256, 512) and the quad-shuffle
    ones with the fused column pass (B = 1024, 2048)."""
    iters = 3
    with m2.Engine(p, mode, path=m2.PATH_LARGE) as e:
        info = e.info()
        assert info.rows == 256 and info.cols_per_cta == 4
        e.iterate(iters)
        got = e.digits()
    o = oracle_mod.Oracle(p, mode)
    o.iterate(iters)
    _cmp(got, o.digits(), f"large p={p} mode={mode}")


@pytest.mark.parametrize("p", [9941, 44497, 132049])
def test_paths_agree(m2, p):
    """The one-CTA path and the three-pass path give the same state."""
    with m2.Engine(p, m2.MODE_PRP, path=m2.PATH_SMALL) as a, m2.Engine(p, m2.MODE_PRP, path=m2.PATH_LARGE) as b:
        for _ in range(3):
            a.iterate(500)
            b.iterate(500)
            _cmp(a.digits(), b.digits(), f"paths p={p}")


def test_contexts_of_different_plans_coexist(m2, oracle_mod):
    """Kernel launch limits are per kernel, shared by every context: a context
    created later with a smaller plan must not break an earlier larger one."""
    with m2.Engine(2976221, 1, path=m2.PATH_LARGE) as big, m2.Engine(756839, 1, path=m2.PATH_LARGE) as small:
        small.iterate(5)
        big.iterate(5)
        o = oracle_mod.Oracle(2976221, 1)
        o.iterate(5)
        _cmp(big.digits(), o.digits(), "earlier, larger plan")
        o2 = oracle_mod.Oracle(756839, 1)
        o2.iterate(5)
        _cmp(small.digits(), o2.digits(), "later, smaller plan")


@pytest.mark.parametrize("p", [5, 7, 13, 31, 61, 89, 107, 127, 521, 607, 1279])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_gf61_only_full_runs_exact(m2, oracle_mod, p, mode):
    """GF(P61^2)-only transforms (the GF61 prototype's size rule): full runs give
    the exact residue and verdict."""
    with m2.Engine(p, mode, fields=m2.FIELDS_GF61) as e:
        assert e.info().fields == m2.FIELDS_GF61 and e.info().ln == m2.layout(p, m2.FIELDS_GF61)[0]
        iters = m2.total_iterations(p, mode)
        e.iterate(iters)
        want = oracle_mod.python_chain(p, mode, iters) % ((1 << p) - 1)
        assert e.res64() == want & ((1 << 64) - 1)
        assert e.verdict() == (want == {0: 0, 1: 9 % ((1 << p) - 1), 2: 3 % ((1 << p) - 1)}[mode])


@pytest.mark.parametrize("p", [9941, 44497, 132049, 216091, 376831])
@pytest.mark.parametrize("mode", [0, 1])
def test_gf61_only_matches_dual_fields(m2, p, mode):
    """Same residues as the dual-field engine, in a layout of as many or more digits."""
    with m2.Engine(p, mode, fields=m2.FIELDS_GF61) as a, m2.Engine(p, mode) as b:
        assert a.info().n >= b.info().n
        for _ in range(3):
            a.iterate(700)
            b.iterate(700)
            assert a.res64() == b.res64(), p


@pytest.mark.parametrize("p,n", [(2976221, 1 << 18), (18874367, 1 << 20), (36700159, 1 << 21)])
def test_gf61_only_three_pass_matches_dual_fields(m2, p, n):
    """GF(P61^2)-only layouts on the three-pass path (the kernel build without
    the GF(P31^2) half): the generic kernels (n = 2^18: 256 x 512) and the
    quad-shuffle ones with the cooperative fused column pass (n = 2^20:
    256 x 2048; n = 2^21: 1024 x 1024 with the phase barrier) give the
    dual-field engine's residues."""
    with m2.Engine(p, 1, fields=m2.FIELDS_GF61) as a, m2.Engine(p, 1) as b:
        assert a.info().path == m2.PATH_LARGE and a.info().n == n and b.info().n == n // 2
        for _ in range(2):
            a.iterate(500)
            b.iterate(500)
            assert a.res64() == b.res64(), p


def test_gf61_only_n2_22_against_gmp(m2):
    """p = 57885161 in the GF(P61^2)-only layout (n = 2^22, the fused column pass
    by arrival ticket): PRP and LL residues at 1000 equal GMP's."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "large.json")) as f:
        g = json.load(f)["57885161"]
    for mode, name in ((1, "prp"), (0, "ll")):
        with m2.Engine(57885161, mode, fields=m2.FIELDS_GF61) as e:
            assert e.info().n == 1 << 22 and e.info().fused_cols == 1
            e.iterate(1000)
            assert f"{e.res64():016x}" == g[name]["1000"], name


# cooperative launch (n = 2^19), cooperative with the phase barrier (n = 2^21), groups by arrival ticket (n = 2^22)
@pytest.mark.parametrize("p", [18874367, 57885161, 115640321])
def test_fused_wait_runs_out_and_reports_timeout(m2, oracle_mod, p):
    """Failure detection without a GPU fault: the fused column kernel's flag
    wait is made to run out (group 0's epoch raised past anything its
    predecessor writes); the launch completes, m2_sync reports M2_ETIMEOUT, and
    after a reload the context computes correct results again."""
    with m2.Engine(p, 1, path=m2.PATH_LARGE) as e:
        assert e.info().fused_cols == 1
        start = e.digits()
        assert e._L.m2_test_stall_fused(e._h) == 0
        e.iterate(3)                                 # fwd, rows, mid (CTA 0 waits out), rows, mid, rows, inv
        with pytest.raises(m2.M2Error, match=r"\(-4\)"):
            e.sync()
        e.set_digits(start, 0)                       # reload: flags and status reset
        e.iterate(3)
        got = e.digits()
    o = oracle_mod.Oracle(p, 1)
    o.iterate(3)
    _cmp(got, o.digits(), "after the timeout")


@pytest.mark.parametrize("p,cp", [(9941, 16), (44497, 64), (132049, 256), (216091, 1024)])
def test_small_path_carry_blocks_vs_oracle(m2, oracle_mod, p, cp):
    """-B (carry_pairs) on the one-CTA path: fewer, longer carry segments."""
    with m2.Engine(p, 1, path=m2.PATH_SMALL, carry_pairs=cp, fused_middle=1) as e:
        e.iterate(100)
        got = e.digits()
    o = oracle_mod.Oracle(p, 1)
    o.iterate(100)
    _cmp(got, o.digits(), f"small p={p} -B {cp}")


def test_graph_replays_vs_oracle(m2, oracle_mod):
    """m2_iterate replays captured graphs of 500 and of 50 squarings and
    launches the rest directly: 551 = 500 + 50 + 1 and then 1049 = 2 x 500 + 49
    squarings end on the oracle's digits (generic three-pass kernels)."""
    p = 132049
    with m2.Engine(p, 1, path=m2.PATH_LARGE) as e:
        e.iterate(551)
        first = e.digits()
        e.iterate(1049)
        got = e.digits()
    o = oracle_mod.Oracle(p, 1)
    o.iterate(551)
    _cmp(first, o.digits(), f"p={p} after 551")
    o.iterate(1049)
    _cmp(got, o.digits(), f"p={p} after 1600")


def test_graph_replays_match_direct_launches(m2):
    """The quad-shuffle kernels with the cooperative fused column pass (n =
    2^19): 1049 squarings replayed as two graphs of 500 and 49 launched
    directly end on the same digits as the same squarings launched directly
    in runs of 49 or fewer (each run checked against the oracle elsewhere),
    and the launch count follows the replays (2k + 1 kernels per run of k)."""
    p = 18874367
    with m2.Engine(p, 1, path=m2.PATH_LARGE) as a, m2.Engine(p, 1, path=m2.PATH_LARGE) as b:
        assert a.info().fused_cols == 1
        assert a.launches_for(1049) == 2 * (2 * 500 + 1) + (2 * 49 + 1)
        assert a.launches_for(551) == (2 * 500 + 1) + (2 * 50 + 1) + (2 * 1 + 1)
        a.iterate(1049)
        left = 1049
        while left:
            k = min(left, 49)
            b.iterate(k)
            left -= k
        _cmp(a.digits(), b.digits(), f"p={p} graphs against direct launches")
        assert a.info().iteration == b.info().iteration == 1049


def test_n2_23_vs_oracle_and_largest_size(m2, oracle_mod):
    """n = 2^23, the largest transform the three-pass plan holds (rows of 4096
    elements in one CTA's shared memory; p <= 285212671): a few squarings
    against the oracle, the GF(P61^2)-only layout at the same n against the
    dual engine, and the first exponent past it refused at creation."""
    p = 200000033
    _, n, w = m2.layout(p)
    rng = np.random.default_rng(23)
    start = (rng.integers(0, 1 << 62, n, dtype=np.uint64) & ((np.uint64(1) << w.astype(np.uint64)) - np.uint64(1)))
    with m2.Engine(p, 1) as e:
        assert e.info().n == 1 << 23 and e.info().row_len == 4096
        e.set_digits(start, 0)                # a full-size residue
        e.iterate(3)
        got = e.digits()
    o = oracle_mod.Oracle(p, 1)
    o.set_digits(start, 0)
    o.iterate(3)
    _cmp(got, o.digits(), f"p={p} n=2^23")
    with m2.Engine(115640321, 1, fields=m2.FIELDS_GF61) as a, m2.Engine(115640321, 1) as b:
        assert a.info().n == 1 << 23
        a.iterate(600)
        b.iterate(600)
        assert a.res64() == b.res64()
    with pytest.raises(m2.M2Error, match=r"\(-6\)"):
        m2.Engine(285212677, 1)     # n = 2^24
