"""The serving loop (pps_server_*, continuous batching) on the GPU: each job's
factor list and prime fingerprint from the server, in a mix of concurrent jobs,
must be exactly what the one-job path (and the reference) gives for that job
alone; admission limits and refusals behave as documented."""
from __future__ import annotations

import pytest

from helpers import args_to_spec, lines_of

pytestmark = pytest.mark.gpu


def test_server_mix_equals_jobs_alone(pps, engine):
    jobs, meta = pps.mixed_jobs(seed=11, count=40, scale_p=2e-3, scale_n=2e-2)
    with pps.Server(0) as srv:
        ids = [srv.submit(jp) for jp in jobs]
        results = [srv.wait(i) for i in ids]
        st = srv.stats()
    for (fac, res), jp, m in zip(results, jobs, meta):
        want, wst = engine.run_job(jp)
        assert pps.factors_to_tuples(fac) == pps.factors_to_tuples(want), m
        assert res.primes == wst.primes and res.prime_sum == wst.prime_sum, m
        assert res.status == 0 and res.latency_ms > 0
    assert st.completed == len(jobs) and st.failed == 0 and st.refused == 0
    assert st.queued == 0 and st.running == 0 and st.reserved_bytes == 0
    assert st.waves >= 1 and 0 < st.p50_ms <= st.p99_ms


def test_server_reference_cases(pps, ref_cases):
    names = sorted(k for k in ref_cases if k.startswith("rand"))[:12]
    with pps.Server(0, wave_segments=64) as srv:  # small waves: jobs span several
        ids = {n: srv.submit(pps.normalize(**args_to_spec(ref_cases[n]["args"]))) for n in names}
        for n in names:
            fac, res = srv.wait(ids[n])
            assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(ref_cases[n]["lines"])), n
            assert res.primes == ref_cases[n]["count"], n


def test_server_admission_limits(pps, engine):
    jobs, _ = pps.mixed_jobs(seed=5, count=9, scale_p=1e-3, scale_n=1e-2)
    # two slots: the other jobs wait in the queue and are admitted as slots free
    with pps.Server(0, max_jobs=2) as srv:
        ids = [srv.submit(jp) for jp in jobs]
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st.admitted == len(jobs) and st.completed == len(jobs)
    for (fac, _), jp in zip(got, jobs):
        want, _ = engine.run_job(jp)
        assert pps.factors_to_tuples(fac) == pps.factors_to_tuples(want)


def test_server_refusal_under_small_budget(pps):
    small = pps.normalize(pmin=10**12, pmax=10**12 + 10**6, kmin=1201, kmax=1301, nmin=2000, nmax=2100)
    # about 1.8e5 expected raw candidates: an 11.6 MB reservation against a 1 MiB budget
    big = pps.normalize(pmin=10**12, pmax=10**12 + 10**9, kmin=3, kmax=9999, nmin=1000,
                        nmax=1000000)
    with pps.Server(0, factor_bytes=1 << 20) as srv:
        with pytest.raises(pps.PPSError) as ei:
            srv.submit(big)
        assert ei.value.code == pps.PPS_ERR_INSUFFICIENT_RESOURCE
        jid = srv.submit(small)
        fac, res = srv.wait(jid)
        st = srv.stats()
    assert res.status == 0 and st.refused == 1 and st.completed == 1


def test_server_wait_timeout_poll_and_unknown(pps):
    jp = pps.normalize(pmin=42 * 10**12, pmax=42 * 10**12 + 2 * 10**9, kmin=1201, kmax=9999,
                       nmin=2000000, nmax=3000000)
    with pps.Server(0) as srv:
        jid = srv.submit(jp)
        with pytest.raises(pps.PPSError) as ei:
            srv.wait(jid, timeout=0.0)
        assert ei.value.code == pps.PPS_ERR_TIMEOUT
        assert srv.poll(jid) in (pps.PPS_JOB_QUEUED, pps.PPS_JOB_RUNNING)
        fac, res = srv.wait(jid)
        assert res.status == 0 and res.primes > 0
        with pytest.raises(pps.PPSError) as ei:
            srv.poll(jid)  # released by the wait that returned its result
        assert ei.value.code == pps.PPS_ERR_NOT_FOUND
        with pytest.raises(pps.PPSError) as ei:
            srv.submit(pps.JobParams())  # not normalised
        assert ei.value.code == pps.PPS_ERR_INVALID_PARAM


def test_server_checkpoint_resumes_exactly(pps, engine):
    """A job's checkpoint mid-run (small waves: the boundary moves wave by wave):
    the factors below the boundary plus a job resumed at the boundary give the
    whole result, and the prime fingerprints add up."""
    import time

    jp = pps.normalize(pmin=10**12, pmax=10**12 + 3 * 10**9, kmin=1201, kmax=9999, nmin=2000,
                       nmax=60000)
    with pps.Server(0, wave_segments=256) as srv:
        jid = srv.submit(jp)
        ck = None
        for _ in range(2000):
            fac, c = srv.checkpoint(jid)
            if jp.pmin < c.p < jp.pmax:
                ck = (fac, c)
                break
            time.sleep(0.002)
        full, res = srv.wait(jid)
    assert ck is not None, "no boundary seen while the job ran"
    part, c = ck
    whole = pps.factors_to_tuples(full)
    assert pps.factors_to_tuples(part) == [f for f in whole if f[0] < c.p]
    assert c.factor_count == len(part)
    rest = pps.JobParams(**dict(jp.as_dict(), pmin=c.p))
    tail, tst = engine.run_job(rest)
    assert pps.factors_to_tuples(tail) == [f for f in whole if f[0] >= c.p]
    assert c.count + tst.primes == res.primes
    assert (c.sum + tst.prime_sum) % 2**64 == res.prime_sum
    text = pps.checkpoint_format(c)
    assert pps.checkpoint_parse(text, jp).p == c.p


def test_server_cancel_queued_and_running(pps, engine):
    """A cancelled job (queued or running) ends with PPS_ERR_CANCELLED and frees
    its slot; the server goes on serving, with exact results."""
    long_job = pps.normalize(pmin=42 * 10**12, pmax=42 * 10**12 + 4 * 10**9, kmin=1201, kmax=9999,
                             nmin=2000000, nmax=3000000)
    small = pps.normalize(pmin=10**12, pmax=10**12 + 10**7, kmin=1201, kmax=9999, nmin=2000,
                          nmax=3000)
    with pps.Server(0, max_jobs=1, wave_segments=1024) as srv:
        running = srv.submit(long_job)
        queued = srv.submit(long_job)  # waits: one slot
        srv.cancel(queued)
        assert srv.poll(queued) == pps.PPS_JOB_FAILED
        srv.cancel(running)
        for jid in (queued, running):
            with pytest.raises(pps.PPSError) as ei:
                srv.wait(jid)
            assert ei.value.code == pps.PPS_ERR_CANCELLED
        jid = srv.submit(small)
        fac, res = srv.wait(jid)
        st = srv.stats()
    want, wst = engine.run_job(small)
    assert pps.factors_to_tuples(fac) == pps.factors_to_tuples(want) and res.primes == wst.primes
    assert st.failed == 2 and st.running == 0 and st.queued == 0


def test_server_small_job_overtakes_a_long_one(pps, engine):
    """Waves are cut by walk work: a small job submitted while a long job is
    being walked joins the next wave and finishes long before it, with its
    exact list; the long job's list is exact too."""
    import time

    long_job = pps.normalize(pmin=42 * 10**12, pmax=42 * 10**12 + 3 * 10**9, kmin=1201, kmax=9999,
                             nmin=2000000, nmax=3000000)  # about 3e12 walk steps, over a second of the GPU
    small = pps.normalize(pmin=10**12, pmax=10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    with pps.Server(0, wave_work=2 * 10**10) as srv:
        jl = srv.submit(long_job)
        time.sleep(0.05)  # the long job is in its first waves
        js = srv.submit(small)
        fs, rs = srv.wait(js)
        assert srv.poll(jl) == pps.PPS_JOB_RUNNING
        fl, rl = srv.wait(jl)
    assert rs.latency_ms < rl.latency_ms / 5
    for fac, jp in ((fs, small), (fl, long_job)):
        want, _ = engine.run_job(jp)
        assert pps.factors_to_tuples(fac) == pps.factors_to_tuples(want)
