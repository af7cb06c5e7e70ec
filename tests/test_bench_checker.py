"""The bench's checker leg on the CPU: it passes true factor lists and true
prime fingerprints, and it reports a factor line or a fingerprint planted
wrong (the mistakes are planted in copies of the reference's own lines, on
the CPU).  No GPU."""
from __future__ import annotations

import numpy as np

from helpers import args_to_spec


def _rows(ora, lines):
    a = np.zeros(len(lines), dtype=ora.FACTOR_DTYPE)
    for i, l in enumerate(lines):
        a[i] = ora.parse_line(l)
    return a


def test_checker_passes_true_and_flags_planted(pps, ora, ref_cases):
    import bench

    chk = bench.Checker(nthreads=4)
    good, bad = [], []
    for name in ("large_n_slice0", "large_n_slice1", "many_n_test", "riesel_small"):
        case = ref_cases[name]
        jp = pps.normalize(**args_to_spec(case["args"]))
        rows = _rows(ora, case["lines"])
        good.append((jp, rows))
        chk.fingerprint("true", jp.pmin, jp.pmax, jp.qmax, case["count"], int(case["sum"], 16))
        wrong = rows.copy()
        wrong["n"] += 1
        bad.append((jp, wrong))
        chk.fingerprint("planted", jp.pmin, jp.pmax, jp.qmax, case["count"] + 1, int(case["sum"], 16))
    chk.verify("true", good)
    chk.verify("planted", bad)
    res = chk.results()
    n = sum(len(r) for _, r in good)
    assert res["true"] == {"verified_factors": n, "verify_failures": 0, "fingerprints_checked": 4,
                           "fingerprints_equal": True, "oracle_primes": res["true"]["oracle_primes"]}
    assert res["planted"]["verify_failures"] == n
    assert res["planted"]["fingerprints_equal"] is False
