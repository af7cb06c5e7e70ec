"""The reference's own main.c and sieve.c driving the GPU libraries, on the GPU.

  ppsieve_gpu     main.c + sieve.c + putil.c + clock.c with the GPU plugin
                  (libppsgpu_app.so, include/pps_app.h) in place of pps/app.c +
                  pps/appcu.cu + pps/factor_proth.c;
  tpsieve_gpu     the same with the plugin's twin build (libppsgpu_app_twin.so),
                  the reference's tpsieve;
  ppsieve_dropin  main.c + sieve.c + the reference's unmodified pps/app.c and
                  pps/factor_proth.c, with the GPU library's pps/appcu.h ABI
                  (libppsgpu_appcu.so, include/appcu_compat.h) in place of
                  pps/appcu.cu.

Both are built by `make -C oracle dropin` (from __graft_entry__.build()) out of
the reference's C sources staged in oracle/_ref/src, a git-ignored copy; where
they are not staged these tests skip.  The first case is the reference's own
test, pps/many_n_test.sh:26-34: the command line
`-p42070e9 -P42070050e6 -k 1201 -K 9999 -N 2000000 -z normal -q`, the factor
file's lines sorted and compared with the golden list (the 39 lines the current
reference prints; tests/golden/many_n_test_39.txt).  The others are the small
Proth configuration in full and a Riesel range, against the reference's own
runs (tests/golden/ref_cases.json).  main.c's count=/sum= line must equal the
reference's too."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_OUT = ROOT / "oracle" / "_ref"
GOLDEN = ROOT / "tests" / "golden"
FP_RE = re.compile(r"count=(\d+),sum=0x([0-9a-f]+)")

pytestmark = pytest.mark.gpu

MANY_N = ["-p42070e9", "-P42070050e6", "-k", "1201", "-K", "9999", "-N", "2000000", "-z", "normal", "-q"]


def _binary(name: str) -> Path:
    b = REF_OUT / name
    if not b.exists():
        pytest.skip(f"{name} not built (the reference's C sources are not staged in oracle/_ref/src)")
    return b


def _run(binary: Path, args: list[str], cwd: Path) -> tuple[list[str], re.Match, str]:
    r = subprocess.run([str(binary), *args, "-t1", "-fppfactors.txt"], cwd=cwd, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, (r.returncode, r.stdout[-800:], r.stderr[-800:])
    f = cwd / "ppfactors.txt"
    lines = sorted(l.strip() for l in f.read_text().splitlines() if "|" in l) if f.exists() else []
    return lines, FP_RE.search(r.stderr), r.stderr


@pytest.mark.parametrize("binary", ["ppsieve_gpu", "ppsieve_dropin"])
def test_many_n_test_script(built, binary, tmp_path, ref_cases):
    """pps/many_n_test.sh: sorted factor lines equal the golden list."""
    lines, fp, err = _run(_binary(binary), MANY_N, tmp_path)
    want = [l for l in (GOLDEN / "many_n_test_39.txt").read_text().splitlines() if l]
    assert lines == sorted(want)
    case = ref_cases["many_n_test"]
    assert fp is not None, err[-400:]
    assert int(fp.group(1)) == case["count"] and int(fp.group(2), 16) == int(case["sum"], 16)


@pytest.mark.parametrize("binary", ["ppsieve_gpu", "ppsieve_dropin"])
@pytest.mark.parametrize("name", ["small_proth_full", "riesel_small"])
def test_reference_main_cases(built, binary, name, tmp_path, ref_cases):
    case = ref_cases[name]
    lines, fp, err = _run(_binary(binary), [*case["args"], "-q"], tmp_path)
    assert lines == case["lines"], name
    assert fp is not None, err[-400:]
    assert int(fp.group(1)) == case["count"] and int(fp.group(2), 16) == int(case["sum"], 16)


def test_twin_dropin_matches_reference_twin_build(built, tmp_path):
    """tpsieve_gpu: the reference's main.c and sieve.c with the plugin's twin
    build, against the reference's own twin build (tests/golden/twin_cases.json)."""
    import json

    case = json.loads((GOLDEN / "twin_cases.json").read_text())["twin_small"]
    lines, fp, err = _run(_binary("tpsieve_gpu"), [*case["args"], "-q"], tmp_path)
    assert lines == case["lines"]
    assert fp is not None, err[-400:]
    assert int(fp.group(1)) == case["count"] and int(fp.group(2), 16) == int(case["sum"], 16)


@pytest.mark.parametrize("name", ["twin_in_abcd", "twin_in_newpgen"])
def test_twin_dropin_input_file(built, tmp_path, name):
    """tpsieve_gpu with -i and a file in the twin build's formats, against the
    reference's twin build run with the same file."""
    import json

    case = json.loads((GOLDEN / "twin_input_cases.json").read_text())[name]
    lines, fp, err = _run(_binary("tpsieve_gpu"), [*case["args"], f"-i{GOLDEN / 'inputs' / case['input']}",
                                                   "-q"], tmp_path)
    assert lines == case["lines"]
    assert fp is not None and int(fp.group(1)) == case["count"], err[-400:]
