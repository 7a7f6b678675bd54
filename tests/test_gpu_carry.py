"""Full carry propagation on the device (m2_carry_normalize, and the context
reads built on it) against exact integer arithmetic.

The reference carries with blocks and a serial drain whose top carry re-enters
digit 0 (mersenne2_gpu.cpp:2097-2123, 2922-3004); the expected digits here are
computed from the exact value  sum t_j 2^bitpos_j  mod 2^p - 1."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bitpos(m2, p):
    _, n, w = m2.layout(p)
    return n, w, np.concatenate([[0], np.cumsum(w.astype(np.int64))])


def _value(terms):
    """sum of v << s over (s, v) terms, pairwise (fast for millions of bits)"""
    items = sorted(terms)
    while len(items) > 1:
        nxt = [(items[k][0], items[k][1] + (items[k + 1][1] << (items[k + 1][0] - items[k][0])))
               for k in range(0, len(items) - 1, 2)]
        if len(items) % 2:
            nxt.append(items[-1])
        items = nxt
    s, v = items[0]
    return v << s


def _digits_of(v, p, n, w, bp):
    if n <= 64:
        return np.array([(v >> int(bp[j])) & ((1 << int(w[j])) - 1) for j in range(n)], dtype=np.uint64)
    bits = np.unpackbits(np.frombuffer(v.to_bytes((p + 7) // 8, "little"), dtype=np.uint8), bitorder="little")[:p]
    owner = np.repeat(np.arange(n), w)
    shift = (np.arange(p) - bp[owner]).astype(np.uint64)
    return np.add.reduceat(bits.astype(np.uint64) << shift, bp[:-1].astype(np.int64)).astype(np.uint64)


def _expected(m2, p, digits, carries=None, seg=0):
    n, w, bp = _bitpos(m2, p)
    terms = [(int(bp[j]), int(digits[j])) for j in range(n) if digits[j]]
    if carries is not None:
        terms += [(int(bp[((s + 1) * seg) % n]), int(carries[s])) for s in range(len(carries)) if carries[s]]
    v = (_value(terms) if terms else 0) % ((1 << p) - 1)
    return _digits_of(v, p, n, w, bp)


def _run(m2, p, digits, carries=None, seg=0):
    import torch
    d = torch.tensor(np.asarray(digits, dtype=np.int64), device="cuda")
    c = None if carries is None else torch.tensor(np.asarray(carries, dtype=np.int64), device="cuda")
    out = m2.carry_normalize(p, d, c, seg)
    return out.cpu().numpy().view(np.uint64)


def _balanced(rng, w):
    half = (np.int64(1) << (w.astype(np.int64) - 1))
    return rng.integers(-half, half + 1, dtype=np.int64)


@pytest.mark.parametrize("p", [9941, 132049, 756839, 2976221])
def test_random_relaxed_state_with_segment_carries(m2, p):
    rng = np.random.default_rng(p)
    n, w, _ = _bitpos(m2, p)
    d = _balanced(rng, w)
    seg = 8
    car = rng.integers(-(1 << 40), 1 << 40, size=n // seg, dtype=np.int64)
    got = _run(m2, p, d, car, seg)
    assert np.array_equal(got, _expected(m2, p, d, car, seg))


@pytest.mark.parametrize("p", [4423, 132049, 2976221])
def test_full_length_ripples_and_wrap(m2, p):
    n, w, _ = _bitpos(m2, p)
    mx = (np.uint64(1) << w.astype(np.uint64)) - np.uint64(1)
    cases = {
        "minus one": np.concatenate([[-1], np.zeros(n - 1, dtype=np.int64)]),
        "minus five at the top": np.concatenate([np.zeros(n - 1, dtype=np.int64), [-5]]),
        "all ones plus one": np.concatenate([[int(mx[0]) + 1], mx[1:].astype(np.int64)]),
        "all ones": mx.astype(np.int64),
        "zero": np.zeros(n, dtype=np.int64),
        "top digit overflows into digit 0": np.concatenate([np.zeros(n - 1, dtype=np.int64), [int(mx[-1]) + 3]]),
    }
    for name, d in cases.items():
        got = _run(m2, p, d)
        assert np.array_equal(got, _expected(m2, p, d)), name
    assert not _run(m2, p, cases["all ones"]).any()          # M_p is written as zero


def test_segment_carry_of_the_last_segment_wraps(m2):
    p = 132049
    n, w, _ = _bitpos(m2, p)
    d = np.zeros(n, dtype=np.int64)
    car = np.zeros(n // 16, dtype=np.int64)
    car[-1] = (1 << 45) + 12345        # enters at digit 0
    car[3] = -(1 << 44)
    got = _run(m2, p, d, car, 16)
    assert np.array_equal(got, _expected(m2, p, d, car, 16))


@pytest.mark.parametrize("p", [3, 5, 7, 13, 31, 61, 89, 127])
def test_tiny_exponents(m2, p):
    rng = np.random.default_rng(p)
    n, w, _ = _bitpos(m2, p)
    for _ in range(5):
        d = rng.integers(-(1 << 20), 1 << 20, size=n, dtype=np.int64)
        assert np.array_equal(_run(m2, p, d), _expected(m2, p, d))


def test_state_outside_the_lookahead_range_is_reported(m2):
    p = 2976221                         # digits of 22 / 23 bits
    n, w, _ = _bitpos(m2, p)
    d = np.zeros(n, dtype=np.int64)
    d[7] = 1 << 61                      # chunk 0 carries about 2^39 into chunk 1
    with pytest.raises(m2.M2Error, match=r"\(-5\)"):
        _run(m2, p, d)


@pytest.mark.parametrize("p", [44497, 2976221])
def test_set_digits_round_trip_and_reduction(m2, p):
    rng = np.random.default_rng(7)
    n, w, _ = _bitpos(m2, p)
    canon = np.array([rng.integers(0, 1 << int(x)) for x in w], dtype=np.uint64)
    with m2.Engine(p, m2.MODE_PRP) as e:
        e.set_digits(canon, 5)                                   # canonical: balanced on the device
        assert np.array_equal(e.digits(), canon)
        wide = canon.copy()
        wide[0] += np.uint64(1) << np.uint64(int(w[0]))          # not canonical: reduced on the host
        e.set_digits(wide, 5)
        assert np.array_equal(e.digits(), _expected(m2, p, wide.astype(np.int64)))
