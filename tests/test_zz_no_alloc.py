"""pps_check_primes_noalloc: the allocation-free walk entry point, for callers
that cannot call cudaMalloc (their device memory comes from another
allocator, or they must not allocate while running).  Called through the C ABI
with device buffers this test owns, twice in a row, and checked bit-exactly
against the engine entry point pps_check_primes_device on the same primes.

Collected last on purpose: the entry point keeps a fixed scratch array on the
device for the life of the process."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(pps, jp, d_primes, n, d_out, cap):
    lib = pps.load()
    nout = ctypes.c_uint32()
    rc = lib.pps_check_primes_noalloc(ctypes.byref(jp), ctypes.c_void_p(d_primes), n,
                                      ctypes.c_void_p(d_out), cap, ctypes.byref(nout), None)
    return rc, nout.value


def _noalloc(pps, jp, d_primes, n, d_out, cap):
    rc, n = _call(pps, jp, d_primes, n, d_out, cap)
    assert rc == pps.PPS_OK, pps.load().pps_last_error().decode()
    return n


def _case(pps, ora, spec, cap=4096):
    """The job, its primes on the device, an output buffer, and the engine's
    factor list for the same primes (the existing entry point)."""
    import torch

    jp = pps.normalize(**spec)
    primes = ora.sieve_range(jp.pmin, jp.pmax, jp.qmax)
    d_p = torch.from_numpy(primes.view(np.int64)).to("cuda:0")
    d_out = torch.zeros(cap * 3, dtype=torch.int64, device="cuda:0")  # 24-byte records
    with pps.Engine(0) as eng:
        want, _ = eng.check_primes_device(jp, d_p.data_ptr(), len(primes))
    return jp, d_p, d_out, pps.factors_to_tuples(want)


def _got(pps, d_out, n):
    import torch

    torch.cuda.synchronize()
    return sorted(pps.factors_to_tuples(d_out[: n * 3].cpu().numpy().view(pps.FACTOR_DTYPE)))


def test_noalloc_matches_engine_twice(pps, ora):
    import torch

    spec = dict(pmin=10**12, pmax=10**12 + 10**8, kmin=1201, kmax=9999, nmin=2000, nmax=6000)
    jp = pps.normalize(**spec)
    primes = ora.sieve_range(jp.pmin, jp.pmax, jp.qmax)
    assert len(primes) <= (1 << 24)
    d_p = torch.from_numpy(primes.view(np.int64)).to("cuda:0")
    cap = 4096
    d_out = torch.zeros(cap * 3, dtype=torch.int64, device="cuda:0")  # 24-byte records
    with pps.Engine(0) as eng:
        want, _ = eng.check_primes_device(jp, d_p.data_ptr(), len(primes))
    want = pps.factors_to_tuples(want)
    assert want, "case must produce factors"
    for _ in range(2):
        d_out.zero_()
        n = _noalloc(pps, jp, d_p.data_ptr(), len(primes), d_out.data_ptr(), cap)
        assert _got(pps, d_out, n) == want


def test_noalloc_rejects_oversized_list(pps):
    lib = pps.load()
    jp = pps.normalize(pmin=10**12, pmax=10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000, nmax=3000)
    nout = ctypes.c_uint32()
    too_many = (1 << 24) + 1
    # the size check comes before any device access, so a dummy pointer is never touched
    rc = lib.pps_check_primes_noalloc(ctypes.byref(jp), ctypes.c_void_p(16), too_many,
                                      ctypes.c_void_p(16), 1, ctypes.byref(nout), None)
    assert rc == pps.PPS_ERR_INVALID_PARAM
    assert b"limit" in lib.pps_last_error()


def test_noalloc_short_steps_and_jobs_back_to_back(pps, ora):
    """A job with steps below 32 n (another walk kernel), then a 32-bit-step job,
    then the first again: each matches the engine, so nothing of one call's
    candidates or counts leaks into the next through the shared scratch."""
    a = dict(pmin=2 * 10**11, pmax=2 * 10**11 + 3 * 10**7, kmin=3, kmax=999, nmin=2000, nmax=50000)
    b = dict(pmin=42 * 10**12, pmax=42 * 10**12 + 2 * 10**7, kmin=1201, kmax=9999, nmin=200000,
             nmax=1200000)
    ja, pa, oa, wa = _case(pps, ora, a)
    jb, pb, ob, wb = _case(pps, ora, b)
    assert ja.step < 32 and jb.step == 32
    assert wa and wb
    for jp, d_p, d_out, want in ((ja, pa, oa, wa), (jb, pb, ob, wb), (ja, pa, oa, wa)):
        d_out.zero_()
        n = _noalloc(pps, jp, d_p.data_ptr(), d_p.numel(), d_out.data_ptr(), 4096)
        assert _got(pps, d_out, n) == want


def test_noalloc_output_overflow_is_reported(pps, ora):
    """An output buffer smaller than the factor count: PPS_ERR_OVERFLOW with the
    true count, and the buffer holds a subset of the true factors."""
    spec = dict(pmin=10**12, pmax=10**12 + 10**8, kmin=1201, kmax=9999, nmin=2000, nmax=6000)
    jp, d_p, d_out, want = _case(pps, ora, spec)
    assert len(want) > 2
    rc, n = _call(pps, jp, d_p.data_ptr(), d_p.numel(), d_out.data_ptr(), 2)
    assert rc == pps.PPS_ERR_OVERFLOW
    assert n == len(want)
    assert set(_got(pps, d_out, 2)) <= set(want)


def test_noalloc_candidate_overflow_is_reported(pps, ora):
    """More raw candidates than the scratch holds (about 1.3e5 from 1.5e7 primes
    near 5.5e11 over a million n): PPS_ERR_OVERFLOW, and the same job split into
    smaller prime lists gives the engine's factors."""
    import torch

    spec = dict(pmin=550 * 10**9, pmax=550 * 10**9 + 4 * 10**8, kmin=3, kmax=9999, nmin=2000,
                nmax=1002000)
    jp = pps.normalize(**spec)
    primes = ora.sieve_range(jp.pmin, jp.pmax, jp.qmax)
    raw = 0
    with pps.Engine(0) as eng:
        raw = len(eng.check_primes_raw(jp, primes))
        want, _ = eng.check_primes(jp, primes)
    assert raw > pps.PPS_NOALLOC_MAX_CANDIDATES, raw
    d_p = torch.from_numpy(primes.view(np.int64)).to("cuda:0")
    cap = 1 << 16
    d_out = torch.zeros(cap * 3, dtype=torch.int64, device="cuda:0")
    rc, _ = _call(pps, jp, d_p.data_ptr(), d_p.numel(), d_out.data_ptr(), cap)
    assert rc == pps.PPS_ERR_OVERFLOW
    assert b"candidates" in pps.load().pps_last_error()
    got = []
    parts = 8
    step = (len(primes) + parts - 1) // parts
    for i in range(0, len(primes), step):
        part = d_p[i:i + step]
        n = _noalloc(pps, jp, part.data_ptr(), part.numel(), d_out.data_ptr(), cap)
        got += _got(pps, d_out, n)
    assert sorted(got) == pps.factors_to_tuples(want)
