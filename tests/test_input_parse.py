"""The library's input-file reader (pps_input_read) against the oracle's
restatement of the reference's scan: the same format, side, extents and
completed job for every fixture, and the same refusals.  CPU only (no
device call)."""
from __future__ import annotations

import json
from pathlib import Path

import pytest

from helpers import args_to_spec

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_input_reader_matches_oracle(pps, ora):
    cases = json.loads((GOLDEN / "input_cases.json").read_text())
    for name, case in sorted(cases.items()):
        spec = args_to_spec(case["args"])
        path = GOLDEN / "inputs" / case["input"]
        given = all(spec[f] for f in ("kmin", "kmax", "nmin", "nmax"))
        if case["rc"] != 0:
            with pytest.raises(pps.PPSError) as ei:
                pps.InputFile(path, **spec)
            assert ei.value.code == pps.PPS_ERR_SCANF
            with pytest.raises(ora.OracleError):
                ora.read_input(path, detect=not given)
            continue
        inp = pps.InputFile(path, **spec)
        oi = ora.read_input(path, detect=not given)
        info = inp.info()
        assert info.records == len(oi.records), name
        assert (info.k0, info.k1, info.n0, info.n1) == (oi.k0, oi.k1, oi.n0, oi.n1), name
        assert {"newpgen": 1, "abcd": 2}[oi.format] == info.format and oi.sign == info.sign, name
        ospec = ora.input_spec(oi, spec)
        for f in ("kmin", "kmax", "nmin", "nmax", "sign"):
            assert inp.spec[f] == ospec[f], (name, f)


def test_input_reader_errors(pps, tmp_path):
    with pytest.raises(pps.PPSError) as ei:
        pps.InputFile(tmp_path / "missing.txt", pmin=10**12, pmax=10**12 + 10**6)
    assert ei.value.code == pps.PPS_ERR_FOPEN
    bad = tmp_path / "bad.txt"
    bad.write_text("hello\n1 2\n")
    with pytest.raises(pps.PPSError) as ei:
        pps.InputFile(bad, pmin=10**12, pmax=10**12 + 10**6)
    assert ei.value.code == pps.PPS_ERR_SCANF
    one = tmp_path / "one_line.txt"
    one.write_text("30:P:1:2:1\n")
    with pytest.raises(pps.PPSError) as ei:
        pps.InputFile(one, pmin=10**12, pmax=10**12 + 10**6)
    assert ei.value.code == pps.PPS_ERR_SCANF


def test_twin_input_reader_matches_oracle(pps, ora):
    """The twin build's formats, read for a twin job (sign PPS_SIGN_TWIN)."""
    cases = json.loads((GOLDEN / "twin_input_cases.json").read_text())
    for name, case in sorted(cases.items()):
        spec = dict(args_to_spec(case["args"]), sign=pps.PPS_SIGN_TWIN)
        path = GOLDEN / "inputs" / case["input"]
        given = all(spec[f] for f in ("kmin", "kmax", "nmin", "nmax"))
        if case["rc"] != 0:
            with pytest.raises(pps.PPSError) as ei:
                pps.InputFile(path, **spec)
            assert ei.value.code == pps.PPS_ERR_SCANF
            with pytest.raises(ora.OracleError):
                ora.read_input(path, detect=not given, twin=True)
            continue
        inp = pps.InputFile(path, **spec)
        oi = ora.read_input(path, detect=not given, twin=True)
        info = inp.info()
        k0, k1 = (6 * oi.k0 + 3, 6 * oi.k1 + 3) if oi.format == "abcd_twin" else (oi.k0, oi.k1)
        assert info.records == len(oi.records), name
        assert (info.k0, info.k1, info.n0, info.n1) == (k0, k1, oi.n0, oi.n1), name
        assert {"newpgen": 1, "abcd_twin": 2}[oi.format] == info.format, name
        assert info.sign == oi.sign == pps.PPS_SIGN_TWIN, name
        ospec = ora.input_spec(oi, spec)
        for f in ("kmin", "kmax", "nmin", "nmax", "sign"):
            assert inp.spec[f] == ospec[f], (name, f)
    # a one-side file for a twin job, and a twin file for a one-side job, are refused
    with pytest.raises(pps.PPSError):
        pps.InputFile(GOLDEN / "inputs" / "newpgen_proth.txt", pmin=5 * 10**10, pmax=6 * 10**10,
                      sign=pps.PPS_SIGN_TWIN)
    with pytest.raises(pps.PPSError):
        pps.InputFile(GOLDEN / "inputs" / "twin_newpgen.txt", pmin=5 * 10**10, pmax=6 * 10**10)


def test_twin_abcd_reader_edge_cases(pps, ora, tmp_path):
    """Blank lines between blocks, a block header whose two n differ (the end of
    the file for the reference's scan, pps/app.c:268-270), and text after the
    last block: the library's reader and the oracle's agree on every record."""
    hdr = "ABCD (6*$a+3)*2^{n}+1 & (6*$a+3)*2^{m}-1 [{a}]"
    body = [hdr.format(n=1000, m=1000, a=2), "3", "5", "", hdr.format(n=1001, m=1001, a=0), "1",
            "", "", hdr.format(n=1003, m=1003, a=7), "2", "9"]
    cases = {
        "blank_lines": body,
        "mismatched_header_ends": body[:4] + [hdr.format(n=1001, m=1002, a=0), "1"] + body[8:],
        "trailing_text": body + ["end of file", "4"],
    }
    for name, lines in cases.items():
        path = tmp_path / f"{name}.txt"
        path.write_text("\n".join(lines) + "\n")
        spec = dict(pmin=5 * 10**10, pmax=5 * 10**10 + 10**6, sign=pps.PPS_SIGN_TWIN)
        inp = pps.InputFile(path, **spec)
        oi = ora.read_input(path, twin=True)
        info = inp.info()
        assert info.records == len(oi.records), name
        assert (info.k0, info.k1) == (6 * oi.k0 + 3, 6 * oi.k1 + 3), name
        assert (info.n0, info.n1) == (oi.n0, oi.n1), name
    assert len(ora.read_input(tmp_path / "blank_lines.txt", twin=True).records) == 8
    assert len(ora.read_input(tmp_path / "mismatched_header_ends.txt", twin=True).records) == 3
