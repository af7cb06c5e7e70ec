"""The twin mode (both sides per walk, the reference's SEARCH_TWIN build) of the
oracle, pinned against the reference's own twin build run here
(tests/golden/twin_cases.json, made by tests/golden/make_golden.py twin).
CPU only."""
from __future__ import annotations

import json
import random
from pathlib import Path

import pytest

from helpers import args_to_spec, lines_of

TWIN = 2
GOLDEN = Path(__file__).resolve().parent / "golden" / "twin_cases.json"


@pytest.fixture(scope="module")
def twin_cases():
    return json.loads(GOLDEN.read_text())


def twin_spec(args):
    spec = args_to_spec(args)
    spec["sign"] = TWIN
    return spec


def test_twin_oracle_matches_reference_twin_build(ora, twin_cases):
    total = 0
    for name, case in sorted(twin_cases.items()):
        assert case["rc"] == 0, name
        facs, count, s = ora.run(ora.normalize(**twin_spec(case["args"])))
        assert lines_of(ora.tuples(facs)) == sorted(set(case["lines"])), name
        assert count == case["count"] and s == int(case["sum"], 16), name
        total += len(case["lines"])
    assert total >= 100
    # both sides appear among the reference's lines
    signs = {l[-2:] for c in twin_cases.values() for l in c["lines"]}
    assert signs == {"+1", "-1"}


def test_twin_is_the_union_of_both_sides(ora):
    """Same k/n/p ranges and k residues: the twin list is the Proth list plus
    the Riesel list (no (p, k, n) can divide both k*2^n+1 and k*2^n-1)."""
    rng = random.Random(5)
    for _ in range(6):
        pmin = int(10 ** rng.uniform(12, 14))
        spec = dict(pmin=pmin, pmax=pmin + rng.randrange(10**6, 4 * 10**6), kmin=3,
                    kmax=rng.randrange(500, 9999), nmin=rng.randrange(1000, 5000),
                    nmax=0, kstep=2, koffset=1)
        spec["nmax"] = spec["nmin"] + rng.randrange(1000, 30000)
        tw, cnt, s = ora.run(ora.normalize(**spec, sign=TWIN))
        pr, cnt_p, _ = ora.run(ora.normalize(**spec, sign=1))
        ri, _, _ = ora.run(ora.normalize(**spec, sign=-1))
        assert sorted(ora.tuples(tw)) == sorted(ora.tuples(pr) + ora.tuples(ri)), spec
        assert cnt == cnt_p


def test_twin_parameter_rules(ora):
    """Twin defaults k == 3 (mod 6) (pps/app.c:53-55) and one n less per step
    (pps/appcu.cu:177-180) before the 32-step rule."""
    p = ora.normalize(pmin=10**12, pmax=10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000, nmax=3000,
                      sign=TWIN)
    one = ora.normalize(pmin=10**12, pmax=10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000,
                        nmax=3000, sign=1, kstep=6, koffset=3)
    assert (p.kstep, p.koffset) == (6, 3)
    assert p.kmin % 6 == 3 and p.kmax % 6 == 3 and (p.kmin, p.kmax) == (one.kmin, one.kmax)
    assert p.nstep == one.nstep - 1
