"""The reference's own GPU program on the GB300, checked against this library.

oracle/_ref/ppsieve_ref_cuda is the reference as released for GPUs -- its
main.c, sieve.c, pps/app.c, pps/factor_proth.c and CUDA kernels pps/appcu.cu
-- built for sm_103a by `make -C oracle refcuda` (from __graft_entry__.build())
out of the staged, git-ignored copy of its sources in oracle/_ref/src; where
they are not staged these tests skip.  Its factor lines and count=/sum= line
must equal the golden list of pps/many_n_test.sh and, on a slice of the
large-n Proth range and a Riesel range, this library's results."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import pytest

from helpers import args_to_spec, lines_of

ROOT = Path(__file__).resolve().parent.parent
BIN = ROOT / "oracle" / "_ref" / "ppsieve_ref_cuda"
GOLDEN = ROOT / "tests" / "golden"
FP_RE = re.compile(r"count=(\d+),sum=0x([0-9a-f]+)")

pytestmark = pytest.mark.gpu


def _run(args: list[str], cwd: Path) -> tuple[list[str], int, int]:
    if not BIN.exists():
        pytest.skip("ppsieve_ref_cuda not built (the reference's sources are not staged in oracle/_ref/src)")
    r = subprocess.run([str(BIN), *args, "-t1", "-q", "-fout.txt"], cwd=cwd, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, (r.returncode, r.stderr[-800:])
    m = FP_RE.search(r.stderr)
    assert m, r.stderr[-400:]
    out = cwd / "out.txt"
    lines = sorted(l.strip() for l in out.read_text().splitlines() if "|" in l) if out.exists() else []
    return lines, int(m.group(1)), int(m.group(2), 16)


def test_many_n_test_script(tmp_path):
    """pps/many_n_test.sh's command line: the golden list (39 lines)."""
    lines, _, _ = _run(["-p42070e9", "-P42070050e6", "-k", "1201", "-K", "9999", "-N", "2000000", "-z", "normal"],
                       tmp_path)
    want = [l for l in (GOLDEN / "many_n_test_39.txt").read_text().splitlines() if l]
    assert lines == sorted(want)


def test_large_n_slice_matches_library(pps, engine, tmp_path):
    """[4.2e13, 4.2e13 + 3e8), n in [2e6, 3e6): the same lines, prime count and sum."""
    spec = dict(pmin=42 * 10**12, pmax=42 * 10**12 + 3 * 10**8, kmin=1201, kmax=9999, nmin=2000000, nmax=3000000)
    lines, count, psum = _run([f"-p{spec['pmin']}", f"-P{spec['pmax']}", "-k1201", "-K9999", "-n2000000",
                               "-N3000000"], tmp_path)
    fac, st = engine.run_job(pps.normalize(**spec))
    assert len(lines) > 50
    assert lines == lines_of(pps.factors_to_tuples(fac))
    assert (count, psum) == (st.primes, st.prime_sum)


def test_riesel_range_matches_library(pps, engine, ref_cases, tmp_path):
    case = ref_cases["riesel_small"]
    lines, count, psum = _run(case["args"], tmp_path)
    assert lines == case["lines"]
    fac, st = engine.run_job(pps.normalize(**args_to_spec(case["args"])))
    assert lines == lines_of(pps.factors_to_tuples(fac))
    assert (count, psum) == (st.primes, st.prime_sum)
