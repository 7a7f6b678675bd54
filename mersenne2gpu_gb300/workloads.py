"""Seeded synthetic exponent workloads.

The reference ships no benchmark inputs; its README lists example exponents
(README.md:55-58) and the exponent -> transform table (README.md:69-102).  The
workloads here are drawn deterministically: a 64-bit Mersenne Twister
(MT19937-64, Matsumoto & Nishimura 2000) seeded with the workload index picks
indices into the ascending list of primes of a range.
"""
from __future__ import annotations

import math

import numpy as np

_MASK64 = (1 << 64) - 1


class MT19937_64:
    """MT19937-64 as published by Matsumoto & Nishimura (same output as C++ std::mt19937_64)."""

    _NN, _MM = 312, 156
    _MATRIX_A = 0xB5026F5AA96619E9
    _UM, _LM = 0xFFFFFFFF80000000, 0x7FFFFFFF

    def __init__(self, seed: int = 5489):
        mt = [0] * self._NN
        mt[0] = seed & _MASK64
        for i in range(1, self._NN):
            mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & _MASK64
        self._mt, self._i = mt, self._NN

    def _twist(self) -> None:
        mt, nn, mm = self._mt, self._NN, self._MM
        for i in range(nn):
            x = (mt[i] & self._UM) | (mt[(i + 1) % nn] & self._LM)
            xa = x >> 1
            if x & 1:
                xa ^= self._MATRIX_A
            mt[i] = mt[(i + mm) % nn] ^ xa
        self._i = 0

    def next(self) -> int:
        if self._i >= self._NN:
            self._twist()
        x = self._mt[self._i]
        self._i += 1
        x ^= (x >> 29) & 0x5555555555555555
        x ^= (x << 17) & 0x71D67FFFEDA60000
        x ^= (x << 37) & 0xFFF7EEE000000000
        x ^= x >> 43
        return x & _MASK64

    def uniform(self) -> float:
        """Double in [0, 1) from the top 53 bits."""
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)


def primes_in(lo: int, hi: int) -> np.ndarray:
    """Ascending primes in [lo, hi] (segmented sieve, uint64)."""
    lo = max(lo, 2)
    if hi < lo:
        return np.zeros(0, dtype=np.uint64)
    r = int(math.isqrt(hi))
    small = np.ones(r + 1, dtype=bool)
    small[:2] = False
    for i in range(2, int(math.isqrt(r)) + 1):
        if small[i]:
            small[i * i :: i] = False
    base = np.nonzero(small)[0]
    seg = np.ones(hi - lo + 1, dtype=bool)
    for q in base:
        q = int(q)
        start = max(q * q, ((lo + q - 1) // q) * q)
        seg[start - lo :: q] = False
    return (np.nonzero(seg)[0] + lo).astype(np.uint64)


def uniform_primes(seed: int, lo: int, hi: int, count: int) -> list[int]:
    """`count` primes drawn uniformly (with replacement) from the primes in [lo, hi]."""
    ps = primes_in(lo, hi)
    rng = MT19937_64(seed)
    return [int(ps[rng.next() % len(ps)]) for _ in range(count)]


def log_uniform_primes(seed: int, lo: int, hi: int, count: int) -> list[int]:
    """`count` primes, log-uniform over [lo, hi]: draw x = lo*(hi/lo)^u, take the next prime >= x."""
    ps = primes_in(lo, hi)
    rng = MT19937_64(seed)
    out = []
    for _ in range(count):
        x = lo * math.exp(rng.uniform() * math.log(hi / lo))
        k = int(np.searchsorted(ps, np.uint64(int(x))))
        out.append(int(ps[min(k, len(ps) - 1)]))
    return out


def poisson_arrivals(seed: int, rate_per_s: float, count: int) -> list[float]:
    """Arrival times (s) of a Poisson process of the given rate."""
    rng = MT19937_64(seed)
    t, out = 0.0, []
    for _ in range(count):
        u = rng.uniform()
        t += -math.log(1.0 - u) / rate_per_s
        out.append(t)
    return out


# Workload definitions (seed = workload index).
MID_RANGE = (159763, 319483)      # transform n = 8192
LARGE_N22_RANGE = (73400329, 142606333)  # transform n = 2^22
BATCH_RANGE = (3, 159739)         # transform n = 8 ... 4096
SERVE_RANGE = (1000, 18874367)    # transform n = 32 ... 2^19


def mid_exponents() -> list[int]:
    """20 primes uniform in [159763, 319483] (seed 2)."""
    return uniform_primes(2, *MID_RANGE, 20)


def large_n22_exponent() -> int:
    """One prime uniform in [73400329, 142606333] (seed 3)."""
    return uniform_primes(3, *LARGE_N22_RANGE, 1)[0]


def batch_exponents(count: int = 4096) -> list[int]:
    """`count` primes uniform over the primes in [3, 159739] (seed 4)."""
    return uniform_primes(4, *BATCH_RANGE, count)


def serve_exponents(count: int) -> list[int]:
    """`count` primes log-uniform over [1000, 18874367] (seed 5)."""
    return log_uniform_primes(5, *SERVE_RANGE, count)
