"""Pin the oracle's whole-range checks, used on the GPU's full-size runs:
the prime fingerprint of a range (count and wrapping sum, main.c:1232) against
the reference's own count=/sum= lines and against the oracle's sieve, and the
per-line verification of reported factors against the reference's own output
lines, with mistakes planted in copies of those lines (on the CPU).  CPU only."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from helpers import args_to_spec

GOLDEN = Path(__file__).resolve().parent / "golden"


def _rows(ora, lines):
    t = [ora.parse_line(l) for l in lines]
    a = np.zeros(len(t), dtype=ora.FACTOR_DTYPE)
    for i, (p, k, n, c) in enumerate(t):
        a[i] = (p, k, n, c)
    return a


def test_fingerprint_matches_reference_counts(ora, ref_cases):
    checked = 0
    for name, case in sorted(ref_cases.items()):
        if case["rc"] != 0 or "count" not in case or name.startswith("riesel62"):
            continue
        p = ora.normalize(**args_to_spec(case["args"]))
        cnt, s = ora.fingerprint(p.pmin, p.pmax, p.qmax)
        assert cnt == case["count"] and s == int(case["sum"], 16), name
        checked += 1
    assert checked >= 40


def test_fingerprint_62bit_slice(ora, ref_cases):
    """Sieving primes up to 2^31 (the large-q buckets): the reference's count and
    sum of [2^62 - 2^34, +1e7)."""
    case = ref_cases["riesel62_slice_lo"]
    p = ora.normalize(**args_to_spec(case["args"]))
    assert p.qmax > 2**30
    cnt, s = ora.fingerprint(p.pmin, p.pmax, p.qmax)
    assert cnt == case["count"] and s == int(case["sum"], 16)


def test_fingerprint_matches_sieve(ora):
    rng = np.random.default_rng(7)
    for _ in range(30):
        lo = int(rng.integers(3, 2**42))
        hi = lo + int(rng.integers(1, 4 * 10**6))
        qmax = int(rng.choice([61, 1000, 70000, int(np.sqrt(hi)) + 1]))
        want = ora.sieve_range(lo, hi, qmax)
        cnt, s = ora.fingerprint(lo, hi, qmax, nthreads=int(rng.integers(1, 9)))
        assert cnt == len(want), (lo, hi, qmax)
        assert s == int(want.sum(dtype=np.uint64)), (lo, hi, qmax)


def test_verify_accepts_reference_lines(ora, ref_cases):
    jobs, rows, job_of = [], [], []
    for name, case in sorted(ref_cases.items()):
        if case["rc"] != 0 or not case["lines"]:
            continue
        jobs.append(ora.normalize(**args_to_spec(case["args"])))
        r = _rows(ora, case["lines"])
        rows.append(r)
        job_of += [len(jobs) - 1] * len(r)
    twin = json.loads((GOLDEN / "twin_cases.json").read_text())
    for name, case in sorted(twin.items()):
        if case["rc"] != 0 or not case["lines"]:
            continue
        jobs.append(ora.normalize(**dict(args_to_spec(case["args"]), sign=2)))
        r = _rows(ora, case["lines"])
        rows.append(r)
        job_of += [len(jobs) - 1] * len(r)
    allrows = np.concatenate(rows)
    assert len(allrows) > 200
    fails, bad = ora.verify_factors(jobs, allrows, job_of)
    assert fails == 0, [(allrows[i], bad[i]) for i in np.nonzero(bad)[0][:5]]


def test_verify_flags_planted_mistakes(ora, ref_cases):
    case = ref_cases["large_n_slice0"]
    jp = ora.normalize(**args_to_spec(case["args"]))
    good = _rows(ora, case["lines"])[0]
    p, k, n, c = int(good["p"]), int(good["k"]), int(good["n"]), int(good["c"])
    q = p + 2
    while not ora.is_prime(q):
        q += 2
    planted = [
        ((p + 2 * (1 if not ora.is_prime(p + 2) else 2), k, n, c), 1),  # composite p
        ((q, k, n, c), 32),                      # another prime: not a divisor
        ((p, k + 2, n, c), 32),                  # k shifted
        ((p, k, n + 1, c), 32),                  # n shifted
        ((p, k, n, -c), 16 | 32),                # wrong side
        ((p, 1199, n, c), 4 | 32),               # k below kmin
        ((p, k + 1, n, c), 4 | 32),              # k even
        ((p, k, jp.nmax, c), 8 | 32),            # n == nmax (half-open)
        ((jp.pmax + 11, k, n, c), 2 | 32),       # p beyond the range
    ]
    a = np.zeros(len(planted) + 1, dtype=ora.FACTOR_DTYPE)
    a[0] = (p, k, n, c)
    for i, (row, _) in enumerate(planted):
        a[i + 1] = row
    fails, bad = ora.verify_factors(jp, a)
    assert bad[0] == 0
    assert fails == len(planted)
    for i, (row, bits) in enumerate(planted):
        assert bad[i + 1] & bits == bits, (row, bad[i + 1], bits)


def test_verify_flags_small_factor_lines(ora):
    """pps/oldsort.txt (the older many_n_test.sh output) holds 105 lines with a
    prime factor below 32768 that the current output rule drops: the verifier
    flags exactly those (and only by the output rule)."""
    jp = ora.normalize(pmin=42070 * 10**9, pmax=42070050 * 10**6, kmin=1201, kmax=9999, nmax=2000000)
    old = [l for l in (GOLDEN / "oldsort_144.txt").read_text().splitlines() if l]
    cur = {l for l in (GOLDEN / "many_n_test_39.txt").read_text().splitlines() if l}
    a = _rows(ora, old)
    fails, bad = ora.verify_factors(jp, a)
    assert fails == len(old) - len(cur) == 105
    for line, b in zip(old, bad):
        assert (b != 0) == (line not in cur), line
        assert b in (0, 64), (line, b)
