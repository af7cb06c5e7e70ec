"""Whole configurations on the GPU, checked line by line: the 62-bit Riesel
range [2^62 - 2^34, 2^62) and the large-n Proth range [4.2e13, 4.2e13 + 1e11)
run in full, one 2^31-wide slice per call; every reported factor passes the
oracle's per-line verification (p prime, p | k*2^n+c, k and n in range, the
output rule) and every slice's prime count and sum equal the oracle's sieve.
The full lists are too long for the CPU walk to reproduce; bit-exactness on
slices of both ranges is in test_gpu_parity.py."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPAN = 1 << 31


def _full(pps, ora, engine, spec):
    lists, jobs, slices = [], [], []
    nslices = (spec["pmax"] - spec["pmin"] + SPAN - 1) // SPAN
    for i in range(nslices):
        lo = spec["pmin"] + i * SPAN
        hi = min(spec["pmax"], lo + SPAN)
        jp = pps.normalize(**dict(spec, pmin=lo, pmax=hi))
        fac, st = engine.run_job(jp)
        lists.append(fac)
        jobs.append(ora.normalize(**dict(spec, pmin=lo, pmax=hi)))
        slices.append((lo, hi, jp.qmax, st.primes, st.prime_sum))
    rows = np.concatenate(lists)
    job_of = np.concatenate([np.full(len(f), i, dtype=np.uint32) for i, f in enumerate(lists)])
    fails, bad = ora.verify_factors(jobs, rows, job_of)
    assert fails == 0, [(rows[i], bad[i]) for i in np.nonzero(bad)[0][:5]]
    for lo, hi, qmax, count, psum in slices:
        assert ora.fingerprint(lo, hi, qmax) == (count, psum), (lo, hi)
    return rows, sum(s[3] for s in slices)


def test_riesel62_full_range_verified(pps, ora, engine):
    spec = dict(pmin=(1 << 62) - (1 << 34), pmax=1 << 62, kmin=3, kmax=9999, nmin=100000, nmax=1000000,
                sign=-1)
    rows, primes = _full(pps, ora, engine, spec)
    assert primes > 3.9e8
    assert (rows["c"] == -1).all()


def test_large_n_full_range_verified(pps, ora, engine):
    spec = dict(pmin=42 * 10**12, pmax=42 * 10**12 + 10**11, kmin=1201, kmax=9999, nmin=2000000,
                nmax=3000000)
    rows, primes = _full(pps, ora, engine, spec)
    assert primes > 3.1e9
    # about one factor per 9e4 primes on this range
    assert 25000 < len(rows) < 50000
