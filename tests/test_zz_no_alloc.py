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


def _noalloc(pps, jp, d_primes, n, d_out, cap):
    lib = pps.load()
    nout = ctypes.c_uint32()
    rc = lib.pps_check_primes_noalloc(ctypes.byref(jp), ctypes.c_void_p(d_primes), n,
                                      ctypes.c_void_p(d_out), cap, ctypes.byref(nout), None)
    assert rc == pps.PPS_OK, lib.pps_last_error().decode()
    return nout.value


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
        torch.cuda.synchronize()
        got = d_out[: n * 3].cpu().numpy().view(pps.FACTOR_DTYPE)
        assert sorted(pps.factors_to_tuples(got)) == want


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
