"""The continuous-batching server: each result equals the same test run alone."""
import pytest

pytestmark = pytest.mark.gpu


def test_server_mixed_sizes_match_alone(m2):
    from mersenne2gpu_gb300.serve import Server
    # full small tests (one-CTA path, several transform sizes, both modes) and
    # capped large tests (three-pass path) in one mix
    jobs = [(9941, 1, 0), (9949, 0, 0), (11213, 0, 0), (4423, 1, 0), (21701, 1, 0), (3217, 0, 0),
            (132049, 1, 5000), (756839, 1, 3000), (2976221, 0, 1500), (44497, 1, 0)]
    results = {}
    with Server(budget_bytes=1 << 30, quantum=700) as srv:
        for i, (p, mode, iters) in enumerate(jobs):
            srv.submit(i, p, mode, iters)
        for _ in range(100000):
            srv.step()
            for r in srv.poll():
                results[r.id] = r
            st = srv.stats()
            if st["active"] == 0 and st["queued"] == 0:
                break
    assert len(results) == len(jobs)
    for i, (p, mode, iters) in enumerate(jobs):
        r = results[i]
        assert r.status == 0, (p, r.status)
        with m2.Engine(p, mode) as e:
            e.iterate(r.iters)
            assert r.iters == (iters or m2.total_iterations(p, mode))
            assert e.res64() == r.res64, p
            assert e.verdict() == r.is_prime, p
    assert results[0].is_prime and results[2].is_prime and not results[1].is_prime


def test_server_budget_limits_admission(m2):
    from mersenne2gpu_gb300.serve import Server
    with Server(budget_bytes=13_000, quantum=100) as srv:   # an n = 256 test holds about 3 KB: four fit
        for i in range(12):
            srv.submit(i, 9941, 1, 300)
        srv.step()
        st = srv.stats()
        assert 0 < st["active"] <= 4 and st["queued"] > 0 and st["resident_bytes"] <= 13_000
        # the admitted tests hold their contexts' real allocations, which add up to the resident bytes
        act = srv.active()
        assert len(act) == st["active"] and all(a["device_bytes"] > 0 and a["n"] == 256 for a in act)
        assert sum(a["device_bytes"] for a in act) == st["resident_bytes"]
        assert all(a["done"] + a["inflight"] <= a["total"] == 300 for a in act)
        got = []
        for _ in range(1000):
            srv.step()
            got += srv.poll()
            if len(got) == 12:
                break
        assert len(got) == 12 and len({r.res64 for r in got}) == 1


def test_server_refuses_a_test_larger_than_the_budget(m2):
    """A request that could never fit is refused at submit, so it cannot block
    the FIFO queue behind it."""
    from mersenne2gpu_gb300.serve import Server
    with Server(budget_bytes=13_000, quantum=500) as srv:
        with pytest.raises(m2.M2Error, match=r"\(-2\)"):
            srv.submit(0, 2976221, 1, 100)           # n = 2^17: megabytes
        srv.submit(1, 9941, 1, 0)                    # still served
        got = []
        for _ in range(1000):
            srv.step()
            got += srv.poll()
            if got:
                break
        assert len(got) == 1 and got[0].id == 1 and got[0].is_prime
