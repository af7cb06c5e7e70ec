"""The correctness fallbacks that only a wrong tuning choice reaches, forced on
the GPU through pps_debug_limits and checked bit-exactly against the oracle:

  * a warp whose queue of flagged blocks overflows re-walks its primes (its
    part of the n range) with the exact test at every step -- in the one-job
    queued walks (one and two primes per thread, 32-bit and shorter steps,
    twin) and in the batched walk;
  * a call whose raw-candidate buffer overflows grows it and walks again --
    pps_run_job, pps_check_primes, pps_check_primes_raw and a wave of the
    batched form."""
from __future__ import annotations

import pytest

from helpers import lines_of

pytestmark = pytest.mark.gpu

CASES = [
    # (forced variant, job): 32-bit steps (running-minimum window, single bound,
    # two primes per thread), 27-bit steps, a twin job (26-bit steps)
    (15, dict(pmin=42 * 10**12, pmax=42 * 10**12 + 2 * 10**6, kmin=1201, kmax=9999, nmin=2000000, nmax=2020010)),
    (26, dict(pmin=42 * 10**12, pmax=42 * 10**12 + 2 * 10**6, kmin=1201, kmax=9999, nmin=2000000, nmax=2020010)),
    (16, dict(pmin=(1 << 62) - (1 << 26), pmax=(1 << 62) - (1 << 26) + 10**6, kmin=3, kmax=9999, nmin=100000,
              nmax=130000, sign=-1)),
    (21, dict(pmin=10**12, pmax=10**12 + 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=5000)),
    (24, dict(pmin=10**12, pmax=10**12 + 10**7, kmin=3, kmax=9999, nmin=2000, nmax=3000, sign=2)),
]


@pytest.fixture
def limits(pps):
    lib = pps.load()

    def set_limits(queue: int, first: int) -> None:
        assert lib.pps_debug_limits(queue, first) == pps.PPS_OK

    yield set_limits
    lib.pps_debug_limits(-1, 0)


def _want(ora, spec):
    facs, count, _ = ora.run(ora.normalize(**spec))
    return lines_of(ora.tuples(facs)), count


@pytest.mark.parametrize("queue", [0, 2])
def test_queue_overflow_rewalks_exactly(pps, engine, ora, limits, queue):
    """Warp queue of 0 (every warp with a flagged block or a partial last block
    overflows) or 2 entries, with 1 and 4 threads per prime."""
    limits(queue, 0)
    try:
        for split in (1, 4):
            engine.set_split(split)
            for variant, spec in CASES:
                engine.set_variant(variant)
                want, count = _want(ora, spec)
                if spec.get("sign") == 2:
                    jp = pps.normalize(**spec)
                    fac, st = engine.check_primes(jp, ora.sieve_range(jp.pmin, jp.pmax, jp.qmax))
                else:
                    fac, st = engine.run_job(pps.normalize(**spec))
                assert st.variant == variant
                assert lines_of(pps.factors_to_tuples(fac)) == want, (queue, split, variant)
                assert st.primes == count
    finally:
        engine.set_variant(-1)
        engine.set_split(0)


def test_candidate_buffer_regrows(pps, engine, ora, limits):
    """A first attempt that holds only 3 raw candidates: each call overflows,
    walks again and returns the same list."""
    spec = dict(pmin=10**12, pmax=10**12 + 5 * 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    want, count = _want(ora, spec)
    jp = pps.normalize(**spec)
    primes = ora.sieve_range(jp.pmin, jp.pmax, jp.qmax)
    raw_unlimited = engine.check_primes_raw(jp, primes)
    limits(-1, 3)
    fac, st = engine.run_job(jp)
    assert st.raw_hits > 3
    assert lines_of(pps.factors_to_tuples(fac)) == want and st.primes == count
    fac, _ = engine.check_primes(jp, primes)
    assert lines_of(pps.factors_to_tuples(fac)) == want
    raw = engine.check_primes_raw(jp, primes)
    assert len(raw) > 3 and (raw == raw_unlimited).all()


def test_batched_fallbacks(pps, engine, ora, limits):
    """The batched walk with a warp queue of 1 entry and a first attempt of 5
    raw candidates per wave: every job's list is the oracle's."""
    specs = [dict(s) for _, s in CASES]
    specs.append(dict(pmin=10**12, pmax=10**12 + 2 * 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=4000, sign=-1))
    jobs = [pps.normalize(**s) for s in specs]
    limits(1, 5)
    per, st = engine.run_batch(jobs)
    assert st.raw_hits > 5
    for spec, fac in zip(specs, per):
        want, _ = _want(ora, spec)
        assert lines_of(pps.factors_to_tuples(fac)) == want, spec
