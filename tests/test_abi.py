"""CPU-side checks of the C ABI: the libraries load, export every symbol the
headers declare, normalise parameters exactly like the reference, and fail
cleanly (no exit, an error code) where a GPU is needed but absent."""
from __future__ import annotations

import ctypes
import random
import re
import subprocess
from pathlib import Path

import pytest

from helpers import args_to_spec

ROOT = Path(__file__).resolve().parent.parent
INCLUDE = ROOT / "include"


def _declared(header: Path) -> list[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    externs = re.findall(r"^extern\s+[\w\s\*]+?\b(\w+)\s*;", text, flags=re.M)
    return sorted(set(names + externs))


def _exported(lib: Path) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_libppsgpu_exports_header(built, pps):
    syms = _exported(pps.LIB_PATH)
    want = _declared(INCLUDE / "ppsgpu.h")
    assert "pps_run_job" in want and "pps_normalize" in want
    missing = [s for s in want if s not in syms]
    assert not missing, missing


def test_every_header_is_exported(built, pps):
    libs = [pps.LIB_PATH, pps.COMPAT_LIB_PATH, Path(pps.LIB_PATH).parent / "libppsgpu_app.so"]
    syms = set()
    for lib in libs:
        assert lib.exists(), lib
        syms |= _exported(lib)
    for h in sorted(INCLUDE.glob("*.h")):
        missing = [s for s in _declared(h) if s not in syms]
        assert not missing, (h.name, missing)


def test_no_device_is_an_error_not_an_exit(pps):
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    lib = pps.load()
    h = ctypes.c_void_p()
    rc = lib.pps_engine_create(0, ctypes.byref(h))
    assert rc == pps.PPS_ERR_NO_DEVICE
    assert b"device" in lib.pps_last_error()


def test_normalize_matches_oracle_random(pps, ora):
    rng = random.Random(11)
    agree = 0
    for _ in range(3000):
        spec = dict(
            pmin=rng.choice([0, rng.randrange(3, 1 << 62), int(10 ** rng.uniform(9, 18.6))]),
            pmax=rng.choice([0, rng.randrange(3, 1 << 62), int(10 ** rng.uniform(9, 18.7))]),
            kmin=rng.choice([0, rng.randrange(1, 20000)]),
            kmax=rng.choice([0, rng.randrange(1, 20000), rng.randrange(1, 1 << 40)]),
            nmin=rng.choice([0, rng.randrange(1, 300), rng.randrange(1, 1 << 22)]),
            nmax=rng.choice([0, rng.randrange(1, 1 << 22)]),
            sign=rng.choice([1, -1, 2]),  # 2: twin
            kstep=rng.choice([0, 2, 6]), koffset=rng.choice([0, 1, 3]),
            qmax=rng.choice([0, 0, rng.randrange(61, 1 << 20)]))
        try:
            a = pps.normalize(**spec).as_dict()
        except pps.PPSError as e:
            a = e.code
        try:
            o = ora.normalize(**spec).as_dict()
            o["sign"] = o.pop("c")
        except ora.OracleError as e:
            o = e.args[0]
        if isinstance(a, dict):
            a.pop("step")
            assert isinstance(o, dict), (spec, a, o)
            assert a == o, spec
            agree += 1
        else:
            assert a == o == pps.PPS_ERR_INVALID_PARAM, (spec, a, o)
    # mostly-valid specs: the accepted branch at scale
    for _ in range(2000):
        pmin = int(10 ** rng.uniform(11.5, 18.6))
        kmin = rng.randrange(1, 5000)
        spec = dict(pmin=pmin, pmax=pmin + rng.randrange(1, 10**9), kmin=kmin,
                    kmax=kmin + rng.randrange(0, 10**4), nmin=rng.randrange(0, 1 << 21),
                    nmax=rng.randrange(0, 1 << 22), sign=rng.choice([1, -1]),
                    kstep=rng.choice([0, 2, 6]), koffset=rng.choice([0, 1, 3]))
        try:
            a = pps.normalize(**spec).as_dict()
            a.pop("step")
        except pps.PPSError as e:
            a = e.code
        try:
            o = ora.normalize(**spec).as_dict()
            o["sign"] = o.pop("c")
        except ora.OracleError as e:
            o = e.args[0]
        assert a == o, spec
        agree += isinstance(a, dict)
    assert agree > 500


def test_normalize_reference_fixture_args(pps, ref_cases):
    for name, case in ref_cases.items():
        spec = args_to_spec(case["args"])
        if case["rc"] != 0:
            with pytest.raises(pps.PPSError) as ei:
                pps.normalize(**spec)
            assert ei.value.code == pps.PPS_ERR_INVALID_PARAM
            assert (-178) & 0xFF == case["rc"], name
        else:
            jp = pps.normalize(**spec)
            assert jp.pmin <= jp.pmax


def test_reference_nstep_values(pps):
    # nstep at the three headline configurations (27, 32, 49) and the walk step
    c1 = pps.normalize(pmin=10**12, pmax=10**12 + 2 * 10**8, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    c2 = pps.normalize(pmin=42 * 10**12, pmax=42 * 10**12 + 10**11, kmin=1201, kmax=9999,
                       nmin=2000000, nmax=3000000)
    c3 = pps.normalize(pmin=(1 << 62) - (1 << 34), pmax=1 << 62, kmin=3, kmax=9999, nmin=100000,
                       nmax=1000000, sign=-1)
    assert (c1.nstep, c1.step) == (27, 27)
    assert (c2.nstep, c2.step) == (32, 32)
    assert (c3.nstep, c3.step) == (49, 32)
