"""Stage-by-stage parity of the three-pass squaring (the pattern of the
reference's host self-tests, mersenne2_gpu.cpp:3200-3240 and 3359-3397, which
check each fused kernel on seeded random vectors).  Each stage runs alone
through the m2_test_stage hook and its output is compared with an exact model
of the arithmetic the stage must perform (oracle/stages.py): a wrong stage is
named, where the end-to-end tests only see wrong digits."""
import numpy as np
import pytest


def _first_diff(got, want, R, B, what):
    for e, (g, w) in enumerate(zip(got, want)):
        if g != w:
            raise AssertionError(f"{what}: element {e} (row {e // B} of {R}, column {e % B}): {g} != {w}")


# n = 2^12 (16 rows of 128: a radix-2 level in the rows), 2^13 (64 rows of 64),
# 2^14 (64 rows of 128)
@pytest.mark.gpu
@pytest.mark.parametrize("p", [132049, 216091, 622577])
def test_three_pass_stages_against_exact_model(m2, oracle_mod, p):
    from oracle import stages as S
    _, n, widths = m2.layout(p)
    rng = np.random.default_rng(p)
    canon = np.array([int(rng.integers(0, 1 << int(w))) for w in widths], dtype=np.uint64)
    o = oracle_mod.Oracle(p, 1)
    s61, s31 = o.shifts()
    with m2.Engine(p, 1, path=m2.PATH_LARGE) as e:
        info = e.info()
        R, B = info.rows, info.row_len
        e.set_digits(canon, 0)
        want = S.expected_stages(canon, widths, s61, s31, R, B)
        for stage in (0, 1):
            za, zb = e.test_stage(stage)
            _first_diff(S.canon_field(za, S.P61), want[stage][S.P61], R, B, f"p={p} stage {stage} GF(P61^2)")
            _first_diff(S.canon_field(zb, S.P31), want[stage][S.P31], R, B, f"p={p} stage {stage} GF(P31^2)")
        e.test_stage(2)
        got = e.digits()
    o.set_digits(canon, 0)
    o.iterate(1)
    assert np.array_equal(got, o.digits()), f"p={p} stage 2: digits differ from the oracle's after one squaring"


def test_stage_model_catches_a_planted_fault(oracle_mod):
    """The model's comparison sees a single wrong coordinate (planted in a copy
    of the expected output, on the CPU)."""
    from oracle import stages as S
    a = [(k % S.P31, (3 * k) % S.P31) for k in range(64)]
    res = S.row_residues(a, 8, 8, S.P31)
    bad = list(res)
    bad[13] = ((bad[13][0] + 1) % S.P31, bad[13][1])
    with pytest.raises(AssertionError, match="row 1 of 8, column 5"):
        _first_diff(bad, res, 8, 8, "planted")
