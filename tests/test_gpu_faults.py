"""Allocation failures at every device-buffer allocation of a call, injected on
the host with pps_debug_fail_allocs(skip, 1): the allocator reports failure
before it reaches cudaMalloc, so no kernel is disturbed.  Each failed call must
return PPS_ERR_INSUFFICIENT_RESOURCE, and the same engine or server must then
give the exact result of an undisturbed run.  The sweep moves the failure one
allocation later each time until the call needs no more allocations than it
was allowed, which covers every allocation site on that call's path."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu

MAX_SITES = 64


@pytest.fixture()
def lib(pps):
    lib = pps.load()
    lib.pps_debug_fail_allocs(0, 0)
    yield lib
    lib.pps_debug_fail_allocs(0, 0)


def _sweep(pps, lib, make, call, close, want):
    """Fail allocation number skip+1 of call(make()), for skip = 0, 1, ...;
    returns the number of allocation sites the call went through."""
    for skip in range(MAX_SITES):
        obj = make()
        try:
            lib.pps_debug_fail_allocs(skip, 1)
            err = None
            try:
                got = call(obj)
            except pps.PPSError as e:
                err = e
            injected = lib.pps_debug_fail_allocs(0, 0)
            if err is None:
                # every allocation the call made succeeded: the sweep is complete
                assert injected == 0, "a failed allocation was absorbed silently"
                assert got == want
                return skip
            assert injected == 1, (skip, err)
            assert err.code == pps.PPS_ERR_INSUFFICIENT_RESOURCE, (skip, err)
            # the same object, nothing injected: the exact result
            assert call(obj) == want, skip
        finally:
            close(obj)
    pytest.fail(f"more than {MAX_SITES} allocation sites")


def test_engine_create_failures(pps, lib):
    def call(_):
        with pps.Engine(0):
            return True

    sites = _sweep(pps, lib, lambda: None, call, lambda _: None, True)
    assert sites >= 1


def test_run_job_failures(pps, lib, engine):
    jp = pps.normalize(pmin=10**12, pmax=10**12 + 2 * 10**7, kmin=1201, kmax=9999, nmin=2000,
                       nmax=4000)

    def call(eng):
        fac, st = eng.run_job(jp)
        return pps.factors_to_tuples(fac), st.primes, st.prime_sum

    want = call(engine)
    assert want[0], "case must produce factors"
    sites = _sweep(pps, lib, lambda: pps.Engine(0), call, lambda e: e.close(), want)
    assert sites >= 4  # sieving-prime table, bitmap, prime lists, candidate buffers


def test_run_batch_failures(pps, lib, engine):
    jobs, _ = pps.mixed_jobs(seed=3, count=6, scale_p=1e-3, scale_n=1e-2)

    def call(eng):
        per, st = eng.run_batch(jobs)
        return [pps.factors_to_tuples(f) for f in per], st.primes, st.prime_sum

    want = call(engine)
    sites = _sweep(pps, lib, lambda: pps.Engine(0), call, lambda e: e.close(), want)
    assert sites >= 10  # the batched form's wave buffers and job slots


def test_warm_engine_table_growth_failure(pps, lib, engine):
    """A warm engine whose next job needs a larger sieving-prime table: the
    growth fails, then the retry rebuilds the table and the batched form's
    Barrett constants and graph from it."""
    small = pps.normalize(pmin=2 * 10**11, pmax=2 * 10**11 + 10**7, kmin=3, kmax=999, nmin=5000, nmax=9000)
    large = pps.normalize(pmin=10**15, pmax=10**15 + 10**7, kmin=3, kmax=999, nmin=5000, nmax=9000)

    def one(eng, jp):
        fac, st = eng.run_job(jp)
        return pps.factors_to_tuples(fac), st.primes, st.prime_sum

    def batch(eng, jp):
        per, st = eng.run_batch([jp])
        return pps.factors_to_tuples(per[0]), st.primes, st.prime_sum

    for run in (one, batch):
        want_small, want_large = run(engine, small), run(engine, large)
        with pps.Engine(0) as eng:
            assert run(eng, small) == want_small
            lib.pps_debug_fail_allocs(0, 1)
            with pytest.raises(pps.PPSError) as ei:
                run(eng, large)
            assert lib.pps_debug_fail_allocs(0, 0) == 1
            assert ei.value.code == pps.PPS_ERR_INSUFFICIENT_RESOURCE
            assert run(eng, large) == want_large
            assert run(eng, small) == want_small


def test_server_wave_failure_fails_only_that_wave(pps, lib, engine):
    """The serving loop: a wave whose sieving-prime table cannot grow fails the
    jobs in it with PPS_ERR_INSUFFICIENT_RESOURCE; the server keeps serving and
    the same job submitted again gives the exact result."""
    small = pps.normalize(pmin=2 * 10**11, pmax=2 * 10**11 + 10**7, kmin=3, kmax=999, nmin=5000, nmax=9000)
    large = pps.normalize(pmin=10**15, pmax=10**15 + 10**7, kmin=3, kmax=999, nmin=5000, nmax=9000)
    want, wst = engine.run_job(large)
    with pps.Server(0) as srv:
        fac, res = srv.wait(srv.submit(small))
        assert res.status == 0
        lib.pps_debug_fail_allocs(0, 1)
        jid = srv.submit(large)
        with pytest.raises(pps.PPSError) as ei:
            srv.wait(jid)
        assert lib.pps_debug_fail_allocs(0, 0) == 1
        assert ei.value.code == pps.PPS_ERR_INSUFFICIENT_RESOURCE
        fac, res = srv.wait(srv.submit(large))
        st = srv.stats()
    assert pps.factors_to_tuples(fac) == pps.factors_to_tuples(want)
    assert res.primes == wst.primes and res.prime_sum == wst.prime_sum
    assert st.failed == 1 and st.completed == 2


def test_server_create_failures(pps, lib):
    def call(_):
        with pps.Server(0):
            return True

    sites = _sweep(pps, lib, lambda: None, call, lambda _: None, True)
    assert sites >= 10
