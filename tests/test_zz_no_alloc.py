"""m2_square_noalloc against the regular entry points, through the C ABI.

m2_square_noalloc is for callers that may not allocate device memory (their
framework owns every device buffer, or an allocation would stall a
latency-critical path): they pass a digit buffer they already own and the
engine works in a static device array.  Here the caller's buffer comes from
torch; two calls in a row must leave the same residue, bit for bit, as the
context-based path (m2_create / m2_iterate / m2_get_digits) after the same
numbers of squarings.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M2_EUNSUPPORTED = -6


def _canonical(d: np.ndarray, widths: np.ndarray) -> np.ndarray:
    """Exact carry pass with wrap-around (2^p == 1 mod 2^p - 1); all-ones -> zero."""
    n = len(widths)
    w = [int(x) for x in widths]
    out = [0] * n
    c = 0
    for j in range(n):
        v = int(d[j]) + c
        out[j] = v & ((1 << w[j]) - 1)
        c = v >> w[j]
    for _ in range(64):
        if c == 0:
            break
        for j in range(n):
            v = out[j] + c
            out[j] = v & ((1 << w[j]) - 1)
            c = v >> w[j]
            if c == 0:
                break
    assert c == 0
    if all(out[j] == (1 << w[j]) - 1 for j in range(n)):
        out = [0] * n
    return np.array(out, dtype=np.uint64)


@pytest.mark.parametrize("p,mode", [(1398269, 1), (9437179, 1), (44497, 0), (1398269, 2)])
def test_noalloc_matches_context_path(m2, p, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = m2._lib()
    _, n, widths = m2.layout(p)
    x0 = 4 if mode == 0 else 3
    start = np.zeros(n, dtype=np.int64)
    # x0 spread over the low digits (all widths here exceed 3 bits)
    start[0] = x0
    dev = torch.from_numpy(start).to("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    with m2.Engine(p, mode) as ref:
        for k in (37, 55):   # two calls in a row on the same buffer
            rc = lib.m2_square_noalloc(p, mode, ctypes.c_void_p(dev.data_ptr()), k, ctypes.c_void_p(stream))
            assert rc == 0, m2.M2Error(rc, "m2_square_noalloc")
            ref.iterate(k)
            got = _canonical(dev.cpu().numpy(), widths)
            want = ref.digits()
            assert np.array_equal(got, want), f"p={p}: no-alloc residue differs after {k} more squarings"


@pytest.mark.parametrize("p,mode", [(86243, 1), (756839, 2), (3021377, 0)])
def test_noalloc_accepts_signed_noncanonical_digits(m2, p, mode):
    """Any digits with |d_j| < 2^width_j are a valid input: seeded random signed
    digits over the whole range (including values below -2^(width-1), which the
    entry point must rebalance before its first squaring) against the context
    path loaded with the canonical digits of the same residue."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = m2._lib()
    _, n, widths = m2.layout(p)
    rng = np.random.default_rng(p)
    w = widths.astype(np.int64)
    mag = (rng.random(n) * (2.0 ** w - 1)).astype(np.int64)      # in [0, 2^w - 1)
    sign = rng.integers(0, 2, n) * 2 - 1
    start = mag * sign
    start[:8] = -((1 << w[:8]) - 1)                                 # the extreme negative digits
    canon = _canonical(start, widths)
    dev = torch.from_numpy(start.copy()).to("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    with m2.Engine(p, mode) as ref:
        ref.set_digits(canon, 0)
        for k in (20, 31):
            rc = lib.m2_square_noalloc(p, mode, ctypes.c_void_p(dev.data_ptr()), k, ctypes.c_void_p(stream))
            assert rc == 0, m2.M2Error(rc, "m2_square_noalloc")
            ref.iterate(k)
            got = _canonical(dev.cpu().numpy(), widths)
            assert np.array_equal(got, ref.digits()), f"p={p} mode={mode}: residue differs after {k} more squarings"


def test_noalloc_rejects_out_of_range_sizes(m2):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = m2._lib()
    buf = torch.zeros(16, dtype=torch.int64, device="cuda")
    for p in (9437189, 2203):   # n = 2^19 (over the 8 MiB scratch) and n = 64 (under the plan minimum)
        assert lib.m2_square_noalloc(p, 1, ctypes.c_void_p(buf.data_ptr()), 1, None) == M2_EUNSUPPORTED
