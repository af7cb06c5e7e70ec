"""The batched persistent form (pps_run_batch) on the GPU: every job's factor
list and prime fingerprint must be exactly what the one-job path and the
reference give for that job alone."""
from __future__ import annotations

import pytest

from helpers import args_to_spec, lines_of

pytestmark = pytest.mark.gpu


def test_batch_reference_random_jobs(pps, engine, ref_cases):
    names = sorted(k for k in ref_cases if k.startswith("rand"))
    jobs = [pps.normalize(**args_to_spec(ref_cases[n]["args"])) for n in names]
    per, st = engine.run_batch(jobs)
    pr, _ = engine.batch_job_primes(len(jobs))
    for j, name in enumerate(names):
        case = ref_cases[name]
        assert lines_of(pps.factors_to_tuples(per[j])) == sorted(set(case["lines"])), name
        assert int(pr[j]) == case["count"], name
    assert st.primes == sum(ref_cases[n]["count"] for n in names)


def test_batch_equals_single_jobs_mixed(pps, engine):
    jobs, meta = pps.mixed_jobs(seed=7, count=48, scale_p=2e-3, scale_n=2e-2)
    per, st = engine.run_batch(jobs)
    pr, sm = engine.batch_job_primes(len(jobs))
    total = 0
    for j, jp in enumerate(jobs):
        want, wst = engine.run_job(jp)
        assert pps.factors_to_tuples(per[j]) == pps.factors_to_tuples(want), (j, meta[j])
        assert int(pr[j]) == wst.primes and int(sm[j]) == wst.prime_sum, (j, meta[j])
        total += len(want)
    assert st.factors == total
    assert st.waves >= 1 and st.chunk in (256, 1024, 4096) and st.unroll in (8, 16)
    assert st.primes_per_lane in (1, 2)


def test_batch_repeat_and_degenerate(pps, engine, ora):
    base = [
        dict(pmin=10**12, pmax=10**12 + 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=6000),
        dict(pmin=10**12 + 40, pmax=10**12 + 60, kmin=1201, kmax=9999, nmin=2000, nmax=3000),  # no primes
        dict(pmin=(1 << 62) - 10**6, pmax=1 << 62, kmin=3, kmax=9999, nmin=1000, nmax=1002, sign=-1),
        dict(pmin=42 * 10**12, pmax=42 * 10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000000,
             nmax=2100000),
    ]
    jobs = [pps.normalize(**s) for s in base]
    first, _ = engine.run_batch(jobs)
    second, _ = engine.run_batch(jobs)  # graph replay path
    for j, spec in enumerate(base):
        want, _, _ = ora.run(ora.normalize(**spec))
        assert pps.factors_to_tuples(first[j]) == ora.tuples(want), spec
        assert pps.factors_to_tuples(second[j]) == ora.tuples(want), spec
    # an empty batch is valid
    per, st = engine.run_batch([])
    assert per == [] and st.factors == 0


@pytest.mark.parametrize("unroll,lanes", [(8, 1), (16, 1), (8, 2), (16, 2)])
def test_batch_walk_kernels_match_reference(pps, engine, ref_cases, unroll, lanes):
    """Each batched walk kernel (8- or 16-step blocks, one or two primes per lane
    for the 32-bit-step jobs), forced: every list is the reference's."""
    names = sorted(k for k in ref_cases if k.startswith("rand"))
    extra = ["large_n_slice0", "large_n_slice3", "riesel62_slice_lo", "small_proth_full"]
    names += extra
    jobs = [pps.normalize(**args_to_spec(ref_cases[n]["args"])) for n in names]
    engine.set_batch_walk(unroll, lanes)
    try:
        per, st = engine.run_batch(jobs)
    finally:
        engine.set_batch_walk(0, 0)
    assert (st.unroll, st.primes_per_lane) == (unroll, lanes)
    for j, name in enumerate(names):
        assert lines_of(pps.factors_to_tuples(per[j])) == sorted(set(ref_cases[name]["lines"])), name


@pytest.mark.parametrize("split", [2, 8])
def test_batch_n_parts_match_oracle(pps, engine, ora, ref_cases, split):
    """Each job's n range cut into `split` parts, each part its own work item
    (forced here for every job, the short and the degenerate n ranges too):
    every list is the reference's or the oracle's."""
    names = sorted(k for k in ref_cases if k.startswith("rand"))[:16]
    jobs = [pps.normalize(**args_to_spec(ref_cases[n]["args"])) for n in names]
    extra = [
        dict(pmin=42 * 10**12, pmax=42 * 10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000000, nmax=2100003),
        dict(pmin=(1 << 62) - 10**6, pmax=1 << 62, kmin=3, kmax=9999, nmin=1000, nmax=1002, sign=-1),
        dict(pmin=10**12, pmax=10**12 + 10**7, kmin=3, kmax=9999, nmin=2000, nmax=3000, sign=pps.PPS_SIGN_TWIN),
    ]
    jobs += [pps.normalize(**s) for s in extra]
    engine.set_split(split)
    engine.set_batch_walk(16, 2)  # the two-primes-per-lane walk over the n parts too
    try:
        per, _ = engine.run_batch(jobs)
    finally:
        engine.set_split(0)
        engine.set_batch_walk(0, 0)
    for j, name in enumerate(names):
        assert lines_of(pps.factors_to_tuples(per[j])) == sorted(set(ref_cases[name]["lines"])), name
    for i, spec in enumerate(extra):
        want, _, _ = ora.run(ora.normalize(**spec))
        assert pps.factors_to_tuples(per[len(names) + i]) == ora.tuples(want), spec
