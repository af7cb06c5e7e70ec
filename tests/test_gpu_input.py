"""Input sieve files (-i) as the output rule on the GPU (pps_input_read +
pps_engine_set_input): every reference run with a file is reproduced bit-exactly
(tests/golden/input_cases.json), and the file rule is off again after
pps_engine_set_input(NULL)."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from helpers import args_to_spec, lines_of

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_input_files_match_reference(pps, engine):
    cases = json.loads((GOLDEN / "input_cases.json").read_text())
    total = 0
    try:
        for name, case in sorted(cases.items()):
            spec = args_to_spec(case["args"])
            if case["rc"] != 0:
                with pytest.raises(pps.PPSError) as ei:
                    pps.InputFile(GOLDEN / "inputs" / case["input"], **spec)
                assert ei.value.code == pps.PPS_ERR_SCANF
                continue
            inp = pps.InputFile(GOLDEN / "inputs" / case["input"], **spec)
            engine.set_input(inp)
            fac, st = engine.run_job(pps.normalize(**inp.spec))
            assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(case["lines"])), name
            assert st.primes == case["count"] and st.prime_sum == int(case["sum"], 16), name
            total += len(case["lines"])
    finally:
        engine.set_input(None)
    assert total >= 100


def test_input_rule_is_off_after_reset(pps, engine, ref_cases):
    case = ref_cases["small_proth_full"]
    fac, _ = engine.run_job(pps.normalize(**args_to_spec(case["args"])))
    assert lines_of(pps.factors_to_tuples(fac)) == sorted(set(case["lines"]))


def test_twin_input_files_match_reference(pps, engine, ora):
    """The twin build's formats (tests/golden/twin_input_cases.json: the
    reference's twin build run with -i): pps_run_job takes the one-job twin walk
    when a file is set, and pps_check_primes on the same primes gives the same
    lines."""
    cases = json.loads((GOLDEN / "twin_input_cases.json").read_text())
    total = 0
    try:
        for name, case in sorted(cases.items()):
            spec = dict(args_to_spec(case["args"]), sign=pps.PPS_SIGN_TWIN)
            if case["rc"] != 0:
                with pytest.raises(pps.PPSError) as ei:
                    pps.InputFile(GOLDEN / "inputs" / case["input"], **spec)
                assert ei.value.code == pps.PPS_ERR_SCANF
                continue
            inp = pps.InputFile(GOLDEN / "inputs" / case["input"], **spec)
            engine.set_input(inp)
            jp = pps.normalize(**inp.spec)
            fac, st = engine.run_job(jp)
            want = sorted(set(case["lines"]))
            assert lines_of(pps.factors_to_tuples(fac)) == want, name
            assert st.primes == case["count"] and st.prime_sum == int(case["sum"], 16), name
            assert st.variant in pps.TWIN_VARIANTS, name  # the one-job twin walk
            fac2, _ = engine.check_primes(jp, ora.sieve_range(jp.pmin, jp.pmax, jp.qmax))
            assert lines_of(pps.factors_to_tuples(fac2)) == want, name
            total += len(want)
    finally:
        engine.set_input(None)
    assert total >= 20
