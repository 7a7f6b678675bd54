"""Exact model of what each stage of the engine's three-pass squaring must
compute -- TEST INFRASTRUCTURE ONLY (tests/test_gpu_stages.py).

The reference checks its fused kernels against its own generic chain on
seeded random vectors (mersenne2_gpu.cpp:3200-3240, 3359-3397).  This engine's
transform uses its own roots of unity and plan, so its intermediates are not
the reference's; they are checked against what the mathematics fixes instead:

* input: the n balanced digits d_j of the state, weighted by 2^s_j (the IBDWT
  shifts, mersenne2_gpu.cpp:3921-3944) in each field and packed in pairs,
  a_k = d_2k 2^s_2k + i d_2k+1 2^s_2k+1, as a polynomial A(Z) = sum a_k Z^k of
  degree < h = n/2 over GF(P^2), P = 2^61 - 1 and 2^31 - 1;
* after the forward column pass, row r (R rows of B) holds A(Z) mod
  (Z^B - rho_r), rho_r = w_R^bitrev(r), w_R the engine's primitive R-th root
  (a decimation in frequency with per-block roots leaves the residues at the
  roots in bit-reversed order);
* after the row pass, row r holds 4 B (A'(Z) mod (Z^B - rho_r)), where A' packs
  the weighted cyclic square s = x (*) x of the length-n weighted sequence
  x_j = d_j 2^s_j the same way (the row levels and their inverses scale by B,
  the real-packed centre square by 4);
* the inverse column pass ends the squaring: the oracle's digits.

The engine's roots come from its own generator search (m2_host.cpp gen61 /
gen31): the first a + b i (b, a = 1, 2, ...) whose power of exponent
(P^2 - 1) / 2^k has order 2^k (k = 62, 32), cubed when its order-4 power is -i.
"""
from __future__ import annotations

import numpy as np

P61 = (1 << 61) - 1
P31 = (1 << 31) - 1
_K = {P61: 62, P31: 32}


def cmul(x, y, P):
    return ((x[0] * y[0] - x[1] * y[1]) % P, (x[0] * y[1] + x[1] * y[0]) % P)


def cpow(x, e, P):
    r = (1, 0)
    while e:
        if e & 1:
            r = cmul(r, x, P)
        x = cmul(x, x, P)
        e >>= 1
    return r


_GEN = {}


def generator(P: int):
    """The engine's generator of the Sylow 2-subgroup of GF(P^2)^*."""
    if P not in _GEN:
        k = _K[P]
        e = (P * P - 1) >> k
        for b in range(1, 64):
            for a in range(1, 64):
                y = cpow((a, b), e, P)
                if cpow(y, 1 << (k - 1), P) == (1, 0):
                    continue
                if cpow(y, 1 << (k - 2), P) == (0, P - 1):
                    y = cmul(cmul(y, y, P), y, P)
                _GEN[P] = y
                break
            if P in _GEN:
                break
    return _GEN[P]


def root(P: int, order: int):
    """Primitive root of unity of a power-of-two order (the engine's)."""
    return cpow(generator(P), (1 << _K[P]) // order, P)


def balanced(canon: np.ndarray, widths: np.ndarray) -> list[int]:
    """Digits as the engine balances canonical input (m2_set_digits): a digit at
    or above 2^(w-1) gives 2^w to the next one (the top one to digit 0)."""
    n = len(canon)
    c = [int(x) for x in canon]
    w = [int(x) for x in widths]
    out = []
    for j in range(n):
        v = c[j]
        if w[j] > 0 and c[j] >= 1 << (w[j] - 1):
            v -= 1 << w[j]
        jp = (j - 1) % n
        if w[jp] > 0 and c[jp] >= 1 << (w[jp] - 1):
            v += 1
        out.append(v)
    return out


def weighted(digits: list[int], shifts: np.ndarray, P: int) -> list[int]:
    return [(d % P) * pow(2, int(s), P) % P for d, s in zip(digits, shifts)]


def packed(x: list[int], P: int) -> list[tuple[int, int]]:
    return [(x[2 * k] % P, x[2 * k + 1] % P) for k in range(len(x) // 2)]


def cyclic_square(x: list[int], P: int) -> list[int]:
    """s_j = sum_k x_k x_(j-k mod n) mod P, by one big-integer square
    (Kronecker substitution: every sum fits a slot of 2 log2 P + log2 n + 2 bits)."""
    n = len(x)
    L = 2 * P.bit_length() + n.bit_length() + 2
    X = 0
    for v in reversed(x):
        X = (X << L) | v
    Y = X * X
    mask = (1 << L) - 1
    s = [0] * n
    for j in range(2 * n - 1):
        s[j % n] += (Y >> (L * j)) & mask
    return [v % P for v in s]


def bitrev(i: int, bits: int) -> int:
    r = 0
    for _ in range(bits):
        r = (r << 1) | (i & 1)
        i >>= 1
    return r


def _dft(v: list[tuple[int, int]], w: tuple[int, int], P: int) -> list[tuple[int, int]]:
    """[sum_q v_q w^(q k)] for k < len(v) (len a power of two, w of that order)."""
    n = len(v)
    if n == 1:
        return list(v)
    w2 = cmul(w, w, P)
    E, O = _dft(v[0::2], w2, P), _dft(v[1::2], w2, P)
    out = [None] * n
    t = (1, 0)
    for k in range(n // 2):
        o = cmul(t, O[k], P)
        out[k] = ((E[k][0] + o[0]) % P, (E[k][1] + o[1]) % P)
        out[k + n // 2] = ((E[k][0] - o[0]) % P, (E[k][1] - o[1]) % P)
        t = cmul(t, w, P)
    return out


def row_residues(a: list[tuple[int, int]], R: int, B: int, P: int, scale: int = 1) -> list[tuple[int, int]]:
    """Row r of the result: scale * (A(Z) mod (Z^B - rho_r)), rho_r = w_R^bitrev(r).
    Coefficient m of row r is sum_q a_(m + qB) rho_r^q: column m evaluated at
    every R-th root by a length-R transform, then read in bit-reversed order."""
    bits = R.bit_length() - 1
    wR = root(P, R)
    out = [None] * (R * B)
    for m in range(B):
        col = _dft([a[m + q * B] for q in range(R)], wR, P)
        for r in range(R):
            c = col[bitrev(r, bits)]
            out[r * B + m] = (c[0] * scale % P, c[1] * scale % P)
    return out


def canon_field(v: np.ndarray, P: int) -> list[tuple[int, int]]:
    """(h, 2) engine coordinates (any representative) -> canonical pairs."""
    return [(int(a) % P, int(b) % P) for a, b in v.tolist()]


def expected_stages(canon: np.ndarray, widths: np.ndarray, shifts61: np.ndarray, shifts31: np.ndarray, R: int, B: int):
    """{stage: {P: expected canonical pairs}} for stages 0 and 1 from the
    canonical digits the state was loaded with."""
    d = balanced(canon, widths)
    out = {0: {}, 1: {}}
    for P, sh in ((P61, shifts61), (P31, shifts31)):
        x = weighted(d, sh, P)
        out[0][P] = row_residues(packed(x, P), R, B, P)
        out[1][P] = row_residues(packed(cyclic_square(x, P), P), R, B, P, scale=4 * B)
    return out
