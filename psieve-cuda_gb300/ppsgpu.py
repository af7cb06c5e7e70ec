"""ctypes binding of libppsgpu.so (include/ppsgpu.h) for tests and benchmarks.

The product is the C ABI; this module only marshals arguments.  It never falls
back to anything: if the shared library (or a GPU) is missing, calls raise.

Reference correspondence (Ken-g6/PSieve-CUDA): JobSpec mirrors the options
-p -P -k -K -n -N -R -M -s -Q (main.c:380-398, pps/app.h:47-59); Engine.run_job
is the whole "main.c + sieve.c + pps/app.c + pps/appcu.cu" pipeline for one
range; format_line reproduces the factor-file line of pps/app.c:133.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libppsgpu.so"
COMPAT_LIB_PATH = _PKG / "_build" / "libppsgpu_appcu.so"

PPS_OK = 0
PPS_ERR_INVALID_PARAM = -178
PPS_ERR_INSUFFICIENT_RESOURCE = -198
PPS_ERR_NOT_IMPLEMENTED = -150
PPS_ERR_CUDA = -300
PPS_ERR_NO_DEVICE = -301
PPS_ERR_OVERFLOW = -302
PPS_ERR_TIMEOUT = -303
PPS_ERR_BUSY = -304
PPS_ERR_NOT_FOUND = -305
PPS_ERR_CANCELLED = -306
PPS_NUM_VARIANTS = 18

FACTOR_DTYPE = np.dtype([("p", "<u8"), ("k", "<u8"), ("n", "<u4"), ("c", "<i4")])
HIT_DTYPE = np.dtype([("p", "<u8"), ("k", "<u8"), ("n", "<u4"), ("idx", "<u4")])


class JobSpec(ctypes.Structure):
    _fields_ = [("pmin", ctypes.c_uint64), ("pmax", ctypes.c_uint64),
                ("kmin", ctypes.c_uint64), ("kmax", ctypes.c_uint64),
                ("nmin", ctypes.c_uint32), ("nmax", ctypes.c_uint32),
                ("sign", ctypes.c_int32), ("kstep", ctypes.c_uint32),
                ("koffset", ctypes.c_uint32), ("qmax", ctypes.c_uint32)]


class JobParams(ctypes.Structure):
    _fields_ = [("pmin", ctypes.c_uint64), ("pmax", ctypes.c_uint64),
                ("kmin", ctypes.c_uint64), ("kmax", ctypes.c_uint64),
                ("nmin", ctypes.c_uint32), ("nmax", ctypes.c_uint32),
                ("sign", ctypes.c_int32), ("kstep", ctypes.c_uint32),
                ("koffset", ctypes.c_uint32), ("qmax", ctypes.c_uint32),
                ("nstep", ctypes.c_uint32), ("step", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class JobStats(ctypes.Structure):
    _fields_ = [("primes", ctypes.c_uint64), ("prime_sum", ctypes.c_uint64),
                ("raw_hits", ctypes.c_uint64), ("factors", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("batches", ctypes.c_uint32),
                ("variant", ctypes.c_uint32), ("sieve_ms", ctypes.c_double),
                ("walk_ms", ctypes.c_double), ("filter_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class PPSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ppsgpu error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load libppsgpu.so (built by build.py / __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} not built; run __graft_entry__.build()")
    lib = ctypes.CDLL(str(p))
    P = ctypes.POINTER
    u64p, szp = P(ctypes.c_uint64), P(ctypes.c_size_t)
    sig = {
        "pps_last_error": (ctypes.c_char_p, []),
        "pps_version": (ctypes.c_char_p, []),
        "pps_normalize": (ctypes.c_int, [P(JobSpec), P(JobParams)]),
        "pps_engine_create": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_void_p)]),
        "pps_engine_destroy": (None, [ctypes.c_void_p]),
        "pps_engine_device_bytes": (ctypes.c_uint64, [ctypes.c_void_p]),
        "pps_engine_set_batch_span": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
        "pps_engine_set_variant": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
        "pps_engine_launches": (ctypes.c_uint64, [ctypes.c_void_p]),
        "pps_run_job": (ctypes.c_int, [ctypes.c_void_p, P(JobParams), ctypes.c_void_p,
                                       ctypes.c_size_t, szp, P(JobStats)]),
        "pps_check_primes": (ctypes.c_int, [ctypes.c_void_p, P(JobParams), u64p, ctypes.c_size_t,
                                            ctypes.c_void_p, ctypes.c_size_t, szp, P(JobStats)]),
        "pps_check_primes_raw": (ctypes.c_int, [ctypes.c_void_p, P(JobParams), u64p,
                                                ctypes.c_size_t, ctypes.c_void_p,
                                                ctypes.c_size_t, szp]),
        "pps_check_primes_device": (ctypes.c_int, [ctypes.c_void_p, P(JobParams), ctypes.c_void_p,
                                                   ctypes.c_size_t, ctypes.c_void_p,
                                                   ctypes.c_size_t, szp, P(JobStats)]),
        "pps_sieve_range": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                           ctypes.c_uint32, u64p, ctypes.c_size_t, szp, u64p]),
        "pps_measure_imad_peak": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_double)]),
        "pps_check_primes_noalloc": (ctypes.c_int, [P(JobParams), ctypes.c_void_p, ctypes.c_size_t,
                                                    ctypes.c_void_p, ctypes.c_uint32,
                                                    P(ctypes.c_uint32), ctypes.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib if path is None else _lib
    return lib


def _check(lib, rc: int) -> None:
    if rc != PPS_OK:
        raise PPSError(rc, lib.pps_last_error().decode(errors="replace"))


def normalize(pmin=0, pmax=0, kmin=0, kmax=0, nmin=0, nmax=0, sign=1, kstep=0, koffset=0,
              qmax=0, lib=None) -> JobParams:
    lib = lib or load()
    spec = JobSpec(pmin, pmax, kmin, kmax, nmin, nmax, sign, kstep, koffset, qmax)
    out = JobParams()
    _check(lib, lib.pps_normalize(ctypes.byref(spec), ctypes.byref(out)))
    return out


def format_line(p: int, k: int, n: int, c: int) -> str:
    """The factor-file line of pps/app.c:133: "%llu | %llu*2^%u%+d"."""
    return f"{int(p)} | {int(k)}*2^{int(n)}{int(c):+d}"


def factors_to_tuples(arr: np.ndarray) -> list[tuple[int, int, int, int]]:
    return [(int(r["p"]), int(r["k"]), int(r["n"]), int(r["c"])) for r in arr]


class Engine:
    """One GPU engine (pps_engine_create)."""

    def __init__(self, device: int = 0, lib=None):
        self.lib = lib or load()
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.pps_engine_create(device, ctypes.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            self.lib.pps_engine_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return int(self.lib.pps_engine_launches(self.h))

    @property
    def device_bytes(self) -> int:
        return int(self.lib.pps_engine_device_bytes(self.h))

    def set_batch_span(self, span: int) -> None:
        _check(self.lib, self.lib.pps_engine_set_batch_span(self.h, span))

    def set_variant(self, v: int) -> None:
        _check(self.lib, self.lib.pps_engine_set_variant(self.h, v))

    def _call_factors(self, fn, *args, cap: int = 1 << 16):
        while True:
            out = np.zeros(cap, dtype=FACTOR_DTYPE)
            n = ctypes.c_size_t()
            st = JobStats()
            rc = fn(self.h, *args, out.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(n),
                    ctypes.byref(st))
            if rc == PPS_ERR_OVERFLOW and n.value > cap:
                cap = n.value
                continue
            _check(self.lib, rc)
            return out[: n.value].copy(), st

    def run_job(self, jp: JobParams, cap: int = 1 << 16):
        return self._call_factors(self.lib.pps_run_job, ctypes.byref(jp), cap=cap)

    def check_primes(self, jp: JobParams, primes: np.ndarray, cap: int = 1 << 16):
        P = np.ascontiguousarray(primes, dtype=np.uint64)
        return self._call_factors(self.lib.pps_check_primes, ctypes.byref(jp),
                                  P.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), len(P),
                                  cap=cap)

    def check_primes_device(self, jp: JobParams, dptr: int, n: int, cap: int = 1 << 16):
        return self._call_factors(self.lib.pps_check_primes_device, ctypes.byref(jp),
                                  ctypes.c_void_p(dptr), n, cap=cap)

    def check_primes_raw(self, jp: JobParams, primes: np.ndarray, cap: int = 1 << 16):
        P = np.ascontiguousarray(primes, dtype=np.uint64)
        while True:
            out = np.zeros(cap, dtype=HIT_DTYPE)
            n = ctypes.c_size_t()
            rc = self.lib.pps_check_primes_raw(self.h, ctypes.byref(jp),
                                               P.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                               len(P), out.ctypes.data_as(ctypes.c_void_p), cap,
                                               ctypes.byref(n))
            if rc == PPS_ERR_OVERFLOW and n.value > cap:
                cap = n.value
                continue
            _check(self.lib, rc)
            return out[: n.value].copy()

    def sieve_range(self, lo: int, hi: int, qmax: int = 0, want_primes: bool = False,
                    cap: int | None = None):
        count = ctypes.c_size_t()
        s = ctypes.c_uint64()
        if want_primes:
            cap = cap or max(1024, (hi - lo) // 2 + 64)
            out = np.zeros(cap, dtype=np.uint64)
            _check(self.lib, self.lib.pps_sieve_range(
                self.h, lo, hi, qmax, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), cap,
                ctypes.byref(count), ctypes.byref(s)))
            return out[: count.value].copy(), count.value, s.value
        _check(self.lib, self.lib.pps_sieve_range(self.h, lo, hi, qmax, None, 0,
                                                  ctypes.byref(count), ctypes.byref(s)))
        return None, count.value, s.value

    def imad_peak(self) -> float:
        v = ctypes.c_double()
        _check(self.lib, self.lib.pps_measure_imad_peak(self.h, ctypes.byref(v)))
        return v.value
