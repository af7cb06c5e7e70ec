"""GPU parity: the CUDA path (through the C ABI) against the reference's own
outputs (tests/golden/ref_cases.json, produced by running the reference) and
against the CPU oracle on seeded inputs.  Integer work: bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import args_to_spec, lines_of

pytestmark = pytest.mark.gpu

FAST_CASES = ["small_proth_full", "many_n_test", "large_n_slice0", "large_n_slice1", "large_n_slice2", "large_n_slice3",
              "large_n_slice4", "riesel62_slice_lo", "riesel62_slice_hi", "riesel_small", "kstep6_off3", "qmax_1000",
              "kround", "nmin_auto", "nstep_clamp_ok", "single_k"]


def _gpu_lines(pps, engine, spec):
    jp = pps.normalize(**spec)
    fac, st = engine.run_job(jp)
    return lines_of(pps.factors_to_tuples(fac)), st


def _gpu_lines_primes(pps, engine, ora, spec):
    """Through the prime-list entry point (the one-job walk kernels for every
    side, twin included)."""
    jp = pps.normalize(**spec)
    fac, st = engine.check_primes(jp, ora.sieve_range(jp.pmin, jp.pmax, jp.qmax))
    return lines_of(pps.factors_to_tuples(fac)), st


def ppsgpu_variants() -> int:
    import ppsgpu

    return ppsgpu.PPS_NUM_VARIANTS


@pytest.mark.parametrize("name", FAST_CASES)
def test_reference_cases(pps, engine, ref_cases, name):
    case = ref_cases[name]
    spec = args_to_spec(case["args"])
    got, st = _gpu_lines(pps, engine, spec)
    assert got == sorted(set(case["lines"])), name
    if "count" in case:
        assert st.primes == case["count"]
        assert st.prime_sum == int(case["sum"], 16)


def test_reference_random_jobs(pps, engine, ref_cases):
    names = sorted(k for k in ref_cases if k.startswith("rand"))
    assert names
    for name in names:
        case = ref_cases[name]
        got, st = _gpu_lines(pps, engine, args_to_spec(case["args"]))
        assert got == sorted(set(case["lines"])), name
        assert st.primes == case["count"], name


def test_kat49_planted(pps, engine, kat49):
    for kat in kat49:
        spec = args_to_spec(kat["args"])
        got, _ = _gpu_lines(pps, engine, spec)
        assert got == sorted(set(kat["fixed_lines"])), kat
        want = f"{kat['p']} | {kat['k']}*2^{kat['n']}{kat['c']:+d}"
        # the planted factor is reported unless the output rule drops it
        if want in kat["fixed_lines"]:
            assert want in got


@pytest.mark.parametrize("variant", list(range(ppsgpu_variants())))
def test_every_walk_variant_matches_oracle(pps, engine, ora, variant):
    specs = [
        dict(pmin=10**12, pmax=10**12 + 3 * 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=5000),
        # s = 32 (forced) with the small-p window: p near 2^50, kmax < 2^7
        dict(pmin=1 << 50, pmax=(1 << 50) + 2 * 10**6, kmin=3, kmax=99, nmin=1000, nmax=20000),
        dict(pmin=42 * 10**12, pmax=42 * 10**12 + 3 * 10**6, kmin=1201, kmax=9999, nmin=2000000,
             nmax=2040000),
        dict(pmin=(1 << 62) - (1 << 26), pmax=(1 << 62) - (1 << 26) + 2 * 10**6, kmin=3, kmax=9999,
             nmin=100000, nmax=140000, sign=-1),
    ]
    if variant in pps.TWIN_VARIANTS:  # the twin kernels walk twin jobs (both sides)
        specs = [dict(s, sign=pps.PPS_SIGN_TWIN) for s in specs]
    engine.set_variant(variant)
    ran = 0
    try:
        for spec in specs:
            got, st = _gpu_lines_primes(pps, engine, ora, spec)
            want, cnt, _ = ora.run(ora.normalize(**spec))
            assert got == lines_of(ora.tuples(want)), (variant, spec)
            assert st.primes == cnt
            ran += st.variant == variant
    finally:
        engine.set_variant(-1)
    # every variant is exact for at least one of the jobs, so it really ran
    assert ran >= 1, variant


def test_tuner_keeps_choices_apart_by_pass_rate(pps, ora):
    """A walk variant tuned on one job is not reused for a job of the same step
    class at much smaller p, where its window would pass most steps: at
    p = 1e12 with kmax < 2^14 the plain window K < 2^32 passes 1 step in 256, so
    the choice must be one whose window scales with p (19, 21: K < 2^s; 20: the
    small-p window), and the result exact."""
    a = dict(pmin=10**13, pmax=10**13 + 2**24, kmin=1201, kmax=9999, nmin=200000, nmax=260000)
    b = dict(pmin=10**12, pmax=10**12 + 2**24, kmin=1201, kmax=9999, nmin=200000, nmax=260000)
    with pps.Engine(0) as eng:
        eng.run_job(pps.normalize(**a))
        fac, st = eng.run_job(pps.normalize(**b))
    assert st.variant in (19, 20, 21), st.variant
    want, cnt, _ = ora.run(ora.normalize(**b))
    assert lines_of(pps.factors_to_tuples(fac)) == lines_of(ora.tuples(want))
    assert st.primes == cnt


def test_sieve_matches_oracle(engine, ora):
    rng = np.random.default_rng(5)
    for _ in range(6):
        lo = int(rng.integers(2**33, 2**61))
        hi = lo + int(rng.integers(1, 3 * 10**6))
        qmax = int(np.sqrt(hi)) + 1
        got, n, s = engine.sieve_range(lo, hi, qmax, want_primes=True)
        want = ora.sieve_range(lo, hi, qmax)
        assert n == len(want)
        assert np.array_equal(got, want)
        assert s == int(want.astype(np.uint64).sum(dtype=np.uint64))


def test_sieve_pseudoprime_mode(engine, ora):
    lo, hi, qmax = 10**12, 10**12 + 10**6, 1000
    got, n, _ = engine.sieve_range(lo, hi, qmax, want_primes=True)
    want = ora.sieve_range(lo, hi, qmax)
    assert np.array_equal(got, want)


def test_sieve_base_primes_large_qmax(engine, ora):
    # sieving primes beyond the host seed table are made on the device
    lo = (1 << 62) - 4 * 10**6
    got, n, _ = engine.sieve_range(lo, 1 << 62, 0, want_primes=True)
    want = ora.sieve_range(lo, 1 << 62, int(np.sqrt(float(1 << 62))))
    assert np.array_equal(got, want)


def test_check_host_primes_matches_oracle(pps, engine, ora):
    spec = dict(pmin=10**12, pmax=10**12 + 10**8, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    jp = pps.normalize(**spec)
    primes = ora.sieve_range(spec["pmin"], spec["pmax"], jp.qmax)
    fac, st = engine.check_primes(jp, primes)
    want = ora.walk_list(ora.normalize(**spec), primes)
    assert pps.factors_to_tuples(fac) == ora.tuples(want)
    assert st.primes == len(primes)


def test_raw_hits_cover_factors(pps, engine, ora):
    spec = dict(pmin=10**12, pmax=10**12 + 5 * 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    jp = pps.normalize(**spec)
    primes = ora.sieve_range(spec["pmin"], spec["pmax"], jp.qmax)
    raw = engine.check_primes_raw(jp, primes)
    fac, _ = engine.check_primes(jp, primes)
    rawset = {(int(h["p"]), int(h["k"]), int(h["n"])) for h in raw}
    for f in fac:
        assert (int(f["p"]), int(f["k"]), int(f["n"])) in rawset
    for h in raw:
        p, k, n = int(h["p"]), int(h["k"]), int(h["n"])
        assert primes[int(h["idx"])] == p
        assert ora.kpow_mod(k, n, 1, p) == 0
        assert jp.kmin <= k <= jp.kmax and jp.nmin <= n < jp.nmax


def test_empty_and_degenerate(pps, engine, ora):
    # no primes at all in range
    jp = pps.normalize(pmin=10**12 + 40, pmax=10**12 + 60, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    fac, st = engine.run_job(jp)
    assert len(fac) == 0
    # nmin == nmax: the reference clamps nstep to 1 and then requires 2^63 <= pmin,
    # so an empty n range is always rejected (pps/appcu.cu:160-176)
    with pytest.raises(pps.PPSError) as ei:
        pps.normalize(pmin=10**12, pmax=10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000, nmax=2000)
    assert ei.value.code == pps.PPS_ERR_INVALID_PARAM
    # the shortest valid n range at the top of the p range: nstep clamped to 3
    lo = (1 << 62) - 10**6
    spec = dict(pmin=lo, pmax=1 << 62, kmin=3, kmax=9999, nmin=1000, nmax=1002, sign=-1)
    jp = pps.normalize(**spec)
    assert jp.nstep == 3
    fac, st = engine.run_job(jp)
    want, cnt, _ = ora.run(ora.normalize(**spec))
    assert pps.factors_to_tuples(fac) == ora.tuples(want) and st.primes == cnt
    # empty prime list through the host-list entry point
    fac, st = engine.check_primes(jp, np.zeros(0, dtype=np.uint64))
    assert len(fac) == 0


def test_batch_span_does_not_change_results(pps, engine, ora):
    spec = dict(pmin=10**12, pmax=10**12 + 2 * 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=6000)
    jp = pps.normalize(**spec)
    base, _ = engine.run_job(jp)
    engine.set_batch_span(1 << 21)
    try:
        small, st = engine.run_job(jp)
    finally:
        engine.set_batch_span(1 << 31)
    assert st.batches > 5
    assert np.array_equal(base, small)


def test_large_n_slice_per_line(pps, engine, ora):
    """Size-independent property at a large size: every reported line is a true
    factor with the output rule satisfied, and the prime fingerprint matches the
    oracle's sieve."""
    lo = 42 * 10**12 + 10**10
    spec = dict(pmin=lo, pmax=lo + 2 * 10**8, kmin=1201, kmax=9999, nmin=2000000, nmax=3000000)
    jp = pps.normalize(**spec)
    fac, st = engine.run_job(jp)
    for p, k, n, c in pps.factors_to_tuples(fac):
        assert ora.verify_line(p, k, n, c)
        assert ora.small_factor(k, n, c) == 0
        assert 1201 <= k <= 9999 and 2000000 <= n < 3000000
    primes = ora.sieve_range(lo, lo + 2 * 10**8, jp.qmax)
    assert st.primes == len(primes)
    assert st.prime_sum == int(primes.sum(dtype=np.uint64))


@pytest.mark.parametrize("split", [2, 8])
def test_split_walks_match_oracle(pps, engine, ora, split):
    """Threads per prime: each prime's n range cut into `split` parts walked by
    their own threads (forced here), for each kind of queued walk, against the
    oracle; the job shapes leave parts empty, or holding only the partial last
    block, too."""
    cases = [
        # 32-bit steps, running-minimum window: 156 blocks + 3 steps
        (15, dict(pmin=42 * 10**12, pmax=42 * 10**12 + 3 * 10**6, kmin=1201, kmax=9999, nmin=2000000,
                  nmax=2040010)),
        # 62-bit Riesel, single-bound pre-test: 156 blocks + 2 steps
        (16, dict(pmin=(1 << 62) - (1 << 26), pmax=(1 << 62) - (1 << 26) + 2 * 10**6, kmin=3, kmax=9999,
                  nmin=100000, nmax=140000, sign=-1)),
        # 27-bit steps, window K < 2^s: 14 blocks, no partial one (8 parts: the last is empty)
        (21, dict(pmin=10**12, pmax=10**12 + 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=5000)),
        # a twin job (26-bit steps) through the prime-list path: 4 blocks + 7 steps
        (24, dict(pmin=10**12, pmax=10**12 + 10**7, kmin=3, kmax=9999, nmin=2000, nmax=3000,
                  sign=pps.PPS_SIGN_TWIN)),
    ]
    engine.set_split(split)
    try:
        for variant, spec in cases:
            engine.set_variant(variant)
            if spec.get("sign") == pps.PPS_SIGN_TWIN:
                got, st = _gpu_lines_primes(pps, engine, ora, spec)
            else:
                got, st = _gpu_lines(pps, engine, spec)
            want, cnt, _ = ora.run(ora.normalize(**spec))
            assert (st.variant, st.split) == (variant, split)
            assert got == lines_of(ora.tuples(want)), (split, spec)
            assert st.primes == cnt
    finally:
        engine.set_split(0)
        engine.set_variant(-1)


def test_tuner_splits_small_prime_counts(pps, ref_cases):
    """A job with far fewer primes than the GPU's resident threads (the
    reference's 2e6-wide slice at 4.2e13: 63,903 primes, n over a million):
    the tuner walks each prime with more than one thread, and the list is the
    reference's."""
    case = ref_cases["large_n_slice0"]
    from helpers import args_to_spec

    with pps.Engine(0) as eng:
        fac, st = eng.run_job(pps.normalize(**args_to_spec(case["args"])))
    assert st.split >= 2, st.split
    assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(case["lines"]))
    assert st.primes == case["count"]


def test_check_primes_reads_pinned_list_in_place(pps, engine, ora):
    """pps_check_primes on a page-locked host list (read in place by the walk)
    and on a pageable one (copied first): the same factors, both the oracle's."""
    torch = pytest.importorskip("torch")
    spec = dict(pmin=10**12, pmax=10**12 + 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=200000)
    jp = pps.normalize(**spec)
    primes = ora.sieve_range(jp.pmin, jp.pmax, jp.qmax)
    pin = torch.empty(len(primes), dtype=torch.int64, pin_memory=True)
    pinned = pin.numpy().view(np.uint64)
    pinned[:] = primes
    fac_pin, st_pin = engine.check_primes(jp, pinned)
    fac, st = engine.check_primes(jp, primes)
    assert st_pin.primes == st.primes == len(primes)
    want = lines_of(ora.tuples(ora.walk_list(ora.normalize(**spec), primes)))
    assert len(want) > 0
    assert lines_of(pps.factors_to_tuples(fac_pin)) == lines_of(pps.factors_to_tuples(fac)) == want
