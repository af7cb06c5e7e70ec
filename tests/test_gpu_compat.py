"""The pps/appcu.h compatibility library on the GPU, driven the way the
reference's pps/app.c drives pps/appcu.cu (tests/harness/compat_driver.c).
The per-prime flag bytes must mark exactly the n-subsections in which the
oracle's raw candidates lie (what pps/app.c then re-walks on the CPU)."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HARNESS = ROOT / "tests" / "harness" / "compat_driver.c"

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(pps, tmp_path_factory):
    out = tmp_path_factory.mktemp("compat") / "compat_driver"
    libdir = Path(pps.LIB_PATH).parent
    subprocess.run(["gcc", "-O2", "-std=gnu11", f"-I{ROOT / 'include'}", str(HARNESS), "-o", str(out),
                    f"-L{libdir}", "-lppsgpu_appcu", "-lppsgpu", f"-Wl,-rpath,{libdir}"],
                   check=True)
    return out


def _run(driver, tmp_path, ora, spec, m=0):
    params = ora.normalize(**spec)
    primes = ora.sieve_range(params.pmin, params.pmax, params.qmax)
    pf = tmp_path / "primes.bin"
    primes.astype("<u8").tofile(pf)
    # the reference's app.c computes nstep before cuda_init clamps it (pps/app.c:710-712)
    nstep = 1
    while (params.kmax << nstep) < params.pmin:
        nstep += 1
    r = subprocess.run([str(driver), str(pf), str(params.pmin), str(params.pmax), str(params.kmin),
                        str(params.kmax), str(params.nmin), str(params.nmax), str(params.c),
                        str(nstep), str(m)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert f"nstep {params.nstep}" in lines
    starts = [int(x) for x in next(l for l in lines if l.startswith("starts")).split()[1:]]
    flags = {}
    for l in lines:
        f = l.split()
        if len(f) == 2 and f[0].isdigit():
            flags[int(f[0])] = int(f[1])
    return params, primes, starts, flags


def _expected(ora, params, primes, starts, candidates_primes=None):
    exp = {}
    raw = ora.raw_candidates(params, primes if candidates_primes is None else candidates_primes)
    for p, k, n in raw:
        for j in range(8):
            if starts[j + 1] <= n < starts[j]:
                exp[p] = exp.get(p, 0) | (1 << j)
                break
        else:
            raise AssertionError(("candidate outside every subsection", p, k, n, starts))
    return exp


def test_flags_small_n(driver, tmp_path, ora):
    spec = dict(pmin=10**12, pmax=10**12 + 3 * 10**7, kmin=1201, kmax=9999, nmin=2000, nmax=6000)
    params, primes, starts, flags = _run(driver, tmp_path, ora, spec)
    assert starts[0] == 6000
    exp = _expected(ora, params, primes, starts)
    assert exp, "no candidates: case too small"
    assert flags == exp


def test_flags_large_n_partial_batches(driver, tmp_path, ora):
    # several partial batches (m=1 -> 128*SMs primes per batch), 8 subsections
    spec = dict(pmin=42 * 10**12, pmax=42 * 10**12 + 3 * 10**6, kmin=1201, kmax=9999,
                nmin=2000000, nmax=2400000)
    params, primes, starts, flags = _run(driver, tmp_path, ora, spec, m=1)
    assert len(set(starts)) == 9
    exp = _expected(ora, params, primes, starts)
    assert flags == exp


def test_flags_riesel_nstep49(driver, tmp_path, ora):
    lo = (1 << 62) - (1 << 28)
    spec = dict(pmin=lo, pmax=lo + 2 * 10**6, kmin=3, kmax=9999, nmin=100000, nmax=150000, sign=-1)
    params, primes, starts, flags = _run(driver, tmp_path, ora, spec)
    assert params.nstep == 49
    exp = _expected(ora, params, primes, starts)
    assert flags == exp
