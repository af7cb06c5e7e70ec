"""Twin jobs (both sides from one walk, the reference's SEARCH_TWIN build) on
the GPU: bit-exact against the reference's twin build run here
(tests/golden/twin_cases.json), equal to the union of the two one-sided runs,
and the same through the batched form and the serving loop."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from helpers import args_to_spec, lines_of

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "twin_cases.json"


@pytest.fixture(scope="module")
def twin_cases():
    return json.loads(GOLDEN.read_text())


def twin_params(pps, args):
    spec = args_to_spec(args)
    spec["sign"] = pps.PPS_SIGN_TWIN
    return pps.normalize(**spec)


def test_twin_matches_reference_twin_build(pps, engine, twin_cases):
    for name, case in sorted(twin_cases.items()):
        fac, st = engine.run_job(twin_params(pps, case["args"]))
        assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(case["lines"])), name
        assert st.primes == case["count"] and st.prime_sum == int(case["sum"], 16), name


def test_twin_is_union_of_sides_in_a_batch(pps, engine):
    rng = np.random.default_rng(17)
    jobs, sides = [], []
    for _ in range(12):
        pmin = int(10 ** rng.uniform(12, 17))
        kmin = int(rng.integers(1, 2000)) * 2 + 1
        spec = dict(pmin=pmin, pmax=pmin + int(10 ** rng.uniform(5, 6.5)), kmin=kmin,
                    kmax=kmin + int(10 ** rng.uniform(2, 3.7)), nmin=int(rng.integers(1000, 100000)),
                    kstep=2, koffset=1)
        spec["nmax"] = spec["nmin"] + int(10 ** rng.uniform(2, 4.5))
        try:
            jobs.append(pps.normalize(**spec, sign=pps.PPS_SIGN_TWIN))
        except pps.PPSError:
            continue
        sides.append((pps.normalize(**spec, sign=1), pps.normalize(**spec, sign=-1)))
    assert len(jobs) >= 6
    per, _ = engine.run_batch(jobs)
    for got, (pr, ri) in zip(per, sides):
        want = sorted(pps.factors_to_tuples(engine.run_job(pr)[0]) +
                      pps.factors_to_tuples(engine.run_job(ri)[0]))
        assert pps.factors_to_tuples(got) == want


def test_twin_in_the_serving_loop(pps, engine, twin_cases):
    names = sorted(twin_cases)[:8]
    with pps.Server(0) as srv:
        ids = {n: srv.submit(twin_params(pps, twin_cases[n]["args"])) for n in names}
        for n in names:
            fac, res = srv.wait(ids[n])
            assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(twin_cases[n]["lines"])), n
            assert res.primes == twin_cases[n]["count"], n


def test_twin_on_the_prime_list_path(pps, engine, ora, twin_cases):
    """pps_check_primes with a twin job: the one-job twin kernels (both sides
    per step, the side carried by each candidate)."""
    for name in ("twin_wide_n", "twin_wide_n3", "twin_small"):
        case = twin_cases[name]
        jp = twin_params(pps, case["args"])
        primes = ora.sieve_range(jp.pmin, jp.pmax, jp.qmax)
        fac, st = engine.check_primes(jp, primes)
        assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(case["lines"])), name
        assert st.primes == case["count"] and st.variant >= 22, name
