"""Seeded workloads and the multi-process (replicas) host path on CPU with gloo."""
import os
import socket

import pytest


def test_mt19937_64_reference_output():
    from mersenne2gpu_gb300.workloads import MT19937_64
    r = MT19937_64(5489)
    # first output of std::mt19937_64 with its default seed
    assert r.next() == 14514284786278117030


def test_workloads_in_range_and_deterministic():
    from mersenne2gpu_gb300 import workloads as W
    mid = W.mid_exponents()
    assert len(mid) == 20 and all(159763 <= p <= 319483 for p in mid) and mid == W.mid_exponents()
    big = W.large_n22_exponent()
    assert 73400329 <= big <= 142606333
    b = W.batch_exponents(4096)
    assert len(b) == 4096 and min(b) >= 3 and max(b) <= 159739
    s = W.serve_exponents(100)
    assert all(1000 <= p <= 18874367 for p in s)
    ps = W.primes_in(2, 100)
    assert ps.tolist()[:10] == [2, 3, 5, 7, 11, 13, 17, 19, 23, 29]
    t = W.poisson_arrivals(5, 10.0, 1000)
    assert all(b > a for a, b in zip(t, t[1:])) and 50 < t[-1] < 200


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        out[rank] = d.max(float(rank + 1) * 10.0)
    finally:
        d.close()


def test_bench_replicas_gloo_world2():
    """bench.py's replica path (barrier + max over ranks) with two gloo ranks."""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    if torch.cuda.is_available():
        pytest.skip("CPU-only test")
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == 20.0 and out[1] == 20.0
