"""The app.h plugin (libppsgpu_app.so) on the GPU, driven in main.c's calling
order (tests/harness/plugin_driver.c): the factor file it writes must equal the
reference's own output for the same options."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

from helpers import args_to_spec

ROOT = Path(__file__).resolve().parent.parent
HARNESS = ROOT / "tests" / "harness" / "plugin_driver.c"

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(pps, tmp_path_factory):
    out = tmp_path_factory.mktemp("plugin") / "plugin_driver"
    libdir = Path(pps.LIB_PATH).parent
    subprocess.run(["gcc", "-O2", "-std=gnu11", f"-I{ROOT / 'include'}", str(HARNESS), "-o",
                    str(out), f"-L{libdir}", "-lppsgpu_app", "-lppsgpu", f"-Wl,-rpath,{libdir}"],
                   check=True)
    return out


@pytest.mark.parametrize("name", ["small_proth_full", "many_n_test", "riesel_small", "kstep6_off3",
                                  "large_n_slice2"])
def test_plugin_factor_file(driver, tmp_path, ora, ref_cases, name):
    case = ref_cases[name]
    spec = args_to_spec(case["args"])
    params = ora.normalize(**spec)
    primes = ora.sieve_range(params.pmin, params.pmax, params.qmax)
    pf = tmp_path / "primes.bin"
    primes.astype("<u8").tofile(pf)
    ff = tmp_path / "factors.txt"
    args = [a for a in case["args"] if not a.startswith(("-p", "-P"))]
    r = subprocess.run([str(driver), str(pf), f"-p{params.pmin}", f"-P{params.pmax}", *args,
                        f"-f{ff}", "-m1"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    assert "checkpoint_ok=1" in r.stdout
    lines = sorted(l for l in ff.read_text().splitlines() if "|" in l) if ff.exists() else []
    assert lines == case["lines"]
    assert f"count={case['count']}," in r.stdout
    n = len(lines)
    assert f"Found {n} factor{'' if n == 1 else 's'}" in r.stdout


GOLDEN = ROOT / "tests" / "golden"


@pytest.mark.parametrize("name", ["in_newpgen_proth", "in_abcd_riesel", "in_abcd_riesel_given",
                                  "in_abcd_proth_kmax"])
def test_plugin_input_file(driver, tmp_path, ora, name):
    """-i: the factor file equals the reference's own run with the same file."""
    import json

    import math

    case = json.loads((GOLDEN / "input_cases.json").read_text())[name]
    spec = args_to_spec(case["args"])
    # the first tenth of the fixture's p range (its lines there), to keep the prime file small
    lo, hi = spec["pmin"], spec["pmin"] + (spec["pmax"] - spec["pmin"]) // 10
    primes = ora.sieve_range(lo | 1, hi, math.isqrt(hi))
    pf = tmp_path / "primes.bin"
    primes.astype("<u8").tofile(pf)
    ff = tmp_path / "factors.txt"
    args = [a for a in case["args"] if not a.startswith(("-p", "-P"))]
    r = subprocess.run([str(driver), str(pf), f"-p{lo}", f"-P{hi}", *args,
                        f"-i{GOLDEN / 'inputs' / case['input']}", f"-f{ff}", "-m1"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    lines = sorted(l for l in ff.read_text().splitlines() if "|" in l) if ff.exists() else []
    want = sorted(l for l in case["lines"] if int(l.split("|")[0]) < hi)
    assert lines == want and len(case["lines"]) > 0


def test_plugin_input_file_refused_like_reference(driver, tmp_path):
    """All k/n bounds given: the file is read as ABCD, so a NewPGen file is a
    bad header (the reference exits with ERR_SCANF)."""
    pf = tmp_path / "p.bin"
    pf.write_bytes(b"")
    r = subprocess.run([str(driver), str(pf), "-p50000000000", "-P50001000000", "-k11", "-K61",
                        "-n1200", "-N1800", f"-i{GOLDEN / 'inputs' / 'newpgen_proth.txt'}"],
                       capture_output=True, text=True)
    assert r.returncode == 3 and "bexit(-140)" in r.stderr


def test_plugin_rejects_like_reference(driver, tmp_path):
    pf = tmp_path / "p.bin"
    pf.write_bytes(b"")
    # kmax >= pmin (pps/app.c:671-675)
    r = subprocess.run([str(driver), str(pf), "-p1000000000000", "-P1000000100000", "-k1201",
                        "-K1000000000001", "-n2000", "-N3000"], capture_output=True, text=True)
    assert r.returncode == 3 and "bexit(-178)" in r.stderr
    assert "kmax < pmin" in r.stderr


@pytest.fixture(scope="module")
def twin_driver(pps, tmp_path_factory):
    out = tmp_path_factory.mktemp("plugin_twin") / "plugin_driver_twin"
    libdir = Path(pps.LIB_PATH).parent
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-DPPS_TWIN", f"-I{ROOT / 'include'}", str(HARNESS), "-o",
                    str(out), f"-L{libdir}", "-lppsgpu_app_twin", "-lppsgpu", f"-Wl,-rpath,{libdir}"],
                   check=True)
    return out


@pytest.mark.parametrize("name", ["twin_wide_n", "twin_wide_n3", "twin_small", "twin_all_odd_k"])
def test_twin_plugin_factor_file(twin_driver, tmp_path, ora, name):
    """The twin build of the plugin (tpsieve) against the reference's own twin
    build run with the same options (tests/golden/twin_cases.json)."""
    import json

    case = json.loads((GOLDEN / "twin_cases.json").read_text())[name]
    spec = args_to_spec(case["args"])
    params = ora.normalize(**dict(spec, sign=2))
    primes = ora.sieve_range(params.pmin, params.pmax, params.qmax)
    pf = tmp_path / "primes.bin"
    primes.astype("<u8").tofile(pf)
    ff = tmp_path / "factors.txt"
    args = [a for a in case["args"] if not a.startswith(("-p", "-P"))]
    r = subprocess.run([str(twin_driver), str(pf), f"-p{params.pmin}", f"-P{params.pmax}", *args,
                        f"-f{ff}", "-m1"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    lines = sorted(l for l in ff.read_text().splitlines() if "|" in l) if ff.exists() else []
    assert lines == case["lines"]
    assert f"count={case['count']}," in r.stdout


@pytest.mark.parametrize("name", ["twin_in_newpgen", "twin_in_abcd", "twin_in_abcd_given"])
def test_twin_plugin_input_file(twin_driver, tmp_path, ora, name):
    """-i with the twin build: a file in the twin build's formats is the output
    rule for both sides; the factor file equals the reference's own twin build
    run with the same file (tests/golden/twin_input_cases.json)."""
    import json

    import math

    case = json.loads((GOLDEN / "twin_input_cases.json").read_text())[name]
    spec = args_to_spec(case["args"])
    # the first 4e8 of the fixture's p range (its lines there), to keep the prime file small
    lo, hi = spec["pmin"], spec["pmin"] + 4 * 10**8
    primes = ora.sieve_range(lo | 1, hi, math.isqrt(hi))
    pf = tmp_path / "primes.bin"
    primes.astype("<u8").tofile(pf)
    ff = tmp_path / "factors.txt"
    args = [a for a in case["args"] if not a.startswith(("-p", "-P"))]
    r = subprocess.run([str(twin_driver), str(pf), f"-p{lo}", f"-P{hi}", *args,
                        f"-i{GOLDEN / 'inputs' / case['input']}", f"-f{ff}", "-m1"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    lines = sorted(l for l in ff.read_text().splitlines() if "|" in l) if ff.exists() else []
    want = sorted(l for l in case["lines"] if int(l.split("|")[0]) < hi)
    assert lines == want and {l[-2:] for l in want} == {"+1", "-1"}
