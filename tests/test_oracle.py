"""Pin the CPU oracle: against the reference's own golden vectors
(pps/oldsort.txt, pps/pps_test_ok.txt as committed fixtures derived from them)
and against the reference itself run here (tests/golden/ref_cases.json).
CPU only."""
from __future__ import annotations

import ctypes
from pathlib import Path

import pytest

from helpers import args_to_spec, lines_of

GOLDEN = Path(__file__).resolve().parent / "golden"

CHEAP = ["small_proth_full", "large_n_slice0", "large_n_slice4", "riesel_small", "kstep6_off3", "qmax_1000",
         "kround", "nmin_auto", "nstep_clamp_ok", "single_k"]


@pytest.mark.parametrize("name", CHEAP)
def test_oracle_matches_reference_run(ora, ref_cases, name):
    case = ref_cases[name]
    assert case["rc"] == 0
    facs, count, s = ora.run(ora.normalize(**args_to_spec(case["args"])))
    assert lines_of(ora.tuples(facs)) == sorted(set(case["lines"]))
    assert count == case["count"] and s == int(case["sum"], 16)


def test_oracle_matches_reference_random_jobs(ora, ref_cases):
    names = sorted(k for k in ref_cases if k.startswith("rand"))
    assert len(names) >= 30
    total = 0
    for name in names:
        case = ref_cases[name]
        facs, count, s = ora.run(ora.normalize(**args_to_spec(case["args"])))
        assert lines_of(ora.tuples(facs)) == sorted(set(case["lines"])), name
        assert count == case["count"], name
        total += len(case["lines"])
    assert total > 0


def test_reference_rejections_are_rejections(ora, ref_cases):
    for name, case in ref_cases.items():
        if case["rc"] != 0:
            with pytest.raises(ora.OracleError):
                ora.normalize(**args_to_spec(case["args"]))


def test_no_duplicate_lines_in_reference_runs(ref_cases):
    for name, case in ref_cases.items():
        assert case["unique"] == case["total"], name


def test_many_n_golden(ora):
    """pps/many_n_test.sh range: the 39-line list (the reference golden
    pps/oldsort.txt after the current small-prime output rule)."""
    lines = (GOLDEN / "many_n_test_39.txt").read_text().split("\n")
    lines = [l for l in lines if l]
    assert len(lines) == 39
    params = ora.normalize(pmin=42070 * 10**9, pmax=42070050 * 10**6, kmin=1201, kmax=9999,
                           nmax=2000000)
    assert params.nmin == 76
    for line in lines:
        p, k, n, c = ora.parse_line(line)
        assert ora.verify_line(p, k, n, c)
        assert ora.test_factor(params, k, n, c)
        # the oracle's walk of just this prime reproduces the line
        got = ora.walk_list(params, [p])
        assert line in lines_of(ora.tuples(got))


def test_oldsort_extra_lines_have_small_factors(ora):
    """The 105 lines of pps/oldsort.txt that the current reference no longer
    prints all divide and all have an odd prime factor below 32768."""
    old = [l for l in (GOLDEN / "oldsort_144.txt").read_text().split("\n") if l]
    keep = set(l for l in (GOLDEN / "many_n_test_39.txt").read_text().split("\n") if l)
    assert len(old) == 144
    extra = [l for l in old if l not in keep]
    assert len(extra) == 105
    for line in extra:
        p, k, n, c = ora.parse_line(line)
        assert ora.verify_line(p, k, n, c)
        assert ora.small_factor(k, n, c) != 0
    ok15 = [l for l in (GOLDEN / "pps_test_ok_15.txt").read_text().split("\n") if l]
    assert len(ok15) == 15 and set(ok15) <= keep


def test_small_factor_filter_matches_reference_code(ora):
    """The oracle's small-prime rule against the reference's own compiled
    pps/factor_proth.c (oracle/_ref/libfactor_proth_ref.so)."""
    so = Path(ora.REF_DIR) / "libfactor_proth_ref.so"
    if not so.exists():
        pytest.skip("reference not built here")
    ref = ctypes.CDLL(str(so))
    ref.sieve_small_primes.argtypes = [ctypes.c_int]
    ref.try_all_factors.restype = ctypes.c_int
    ref.try_all_factors.argtypes = [ctypes.c_uint64, ctypes.c_uint, ctypes.c_int]
    ref.sieve_small_primes(11)
    import random

    rng = random.Random(3)
    for _ in range(20000):
        k = rng.randrange(1, 1 << 40) | 1
        n = rng.randrange(64, 1 << 24)
        c = rng.choice([1, -1])
        # try_all_factors covers 11..32767; 3, 5 and 7 are the mod-15 / mod-7 tests
        assert ref.try_all_factors(k, n, c) == ora.small_factor(k, n, c, 11), (k, n, c)


def test_oracle_sieve_fingerprints(ora, ref_cases):
    c1 = ref_cases["small_proth_full"]
    p = ora.normalize(**args_to_spec(c1["args"]))
    primes = ora.sieve_range(p.pmin, p.pmax, p.qmax)
    assert len(primes) == c1["count"] == 7237499
    assert int(primes.sum(dtype="uint64")) == int(c1["sum"], 16) == 0x6473554bc2eb39cd
