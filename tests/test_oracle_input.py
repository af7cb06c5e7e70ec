"""Input sieve files (-i, NewPGen and ABCD formats) as the output rule: the
oracle's restatement of the reference's reading (pps/app.c:190-517) and bitmap
test (pps/app.c:180-183), pinned against the reference run here with -i
(tests/golden/input_cases.json, files in tests/golden/inputs/).  CPU only."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from helpers import args_to_spec, lines_of

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def input_cases():
    return json.loads((GOLDEN / "input_cases.json").read_text())


def oracle_input_job(ora, case):
    spec = args_to_spec(case["args"])
    given = all(spec[f] for f in ("kmin", "kmax", "nmin", "nmax"))
    inp = ora.read_input(GOLDEN / "inputs" / case["input"], detect=not given)
    params = ora.normalize(**ora.input_spec(inp, spec))
    return ora.attach_input(params, ora.input_keys(inp, params))


def test_input_files_match_reference(ora, input_cases):
    total = 0
    for name, case in sorted(input_cases.items()):
        if case["rc"] != 0:
            continue
        facs, count, s = ora.run(oracle_input_job(ora, case))
        assert lines_of(ora.tuples(facs)) == sorted(set(case["lines"])), name
        assert count == case["count"] and s == int(case["sum"], 16), name
        total += len(case["lines"])
    assert total >= 100


def test_input_file_rejections(ora, input_cases):
    for name, case in input_cases.items():
        if case["rc"] == 0:
            continue
        assert case["rc"] == (ora.ERR_SCANF & 0xFF), name
        with pytest.raises(ora.OracleError):
            oracle_input_job(ora, case)


def test_input_file_lines_skip_the_small_prime_filter(ora, input_cases):
    """With a file the reference prints every factor whose (k, n) the file
    holds, small factors or not (pps/app.c:164-183)."""
    some_small = 0
    for case in input_cases.values():
        for line in case["lines"]:
            p, k, n, c = ora.parse_line(line)
            assert ora.verify_line(p, k, n, c)
            some_small += ora.small_factor(k, n, c) != 0
    assert some_small > 0


@pytest.fixture(scope="module")
def twin_input_cases():
    return json.loads((GOLDEN / "twin_input_cases.json").read_text())


def oracle_twin_input_job(ora, case):
    spec = dict(args_to_spec(case["args"]), sign=ora.TWIN)
    given = all(spec[f] for f in ("kmin", "kmax", "nmin", "nmax"))
    inp = ora.read_input(GOLDEN / "inputs" / case["input"], detect=not given, twin=True)
    params = ora.normalize(**ora.input_spec(inp, spec))
    return ora.attach_input(params, ora.input_keys(inp, params))


def test_twin_input_files_match_reference(ora, twin_input_cases):
    """The twin build's formats (NewPGen ":T:", ABCD "(6*$a+3)*2^n+1 & ...-1"):
    the reference's twin build run with -i (tests/golden/twin_input_cases.json)."""
    total = 0
    for name, case in sorted(twin_input_cases.items()):
        if case["rc"] != 0:
            assert case["rc"] == (ora.ERR_SCANF & 0xFF), name
            with pytest.raises(ora.OracleError):
                oracle_twin_input_job(ora, case)
            continue
        facs, count, s = ora.run(oracle_twin_input_job(ora, case))
        assert lines_of(ora.tuples(facs)) == sorted(set(case["lines"])), name
        assert count == case["count"] and s == int(case["sum"], 16), name
        total += len(case["lines"])
    assert total >= 20
    sides = {l.rstrip()[-2:] for c in twin_input_cases.values() for l in c["lines"]}
    assert sides == {"+1", "-1"}
