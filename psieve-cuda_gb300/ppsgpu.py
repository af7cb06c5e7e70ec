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
PPS_NUM_VARIANTS = 31
TWIN_VARIANTS = (22, 23, 24, 25)  # the walks of both sides of a twin job
PPS_SIGN_TWIN = 2  # both sides from one walk (the reference's twin build)
PPS_NOALLOC_MAX_PRIMES = 1 << 24  # per call of pps_check_primes_noalloc
PPS_NOALLOC_MAX_CANDIDATES = 1 << 16

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
                ("total_ms", ctypes.c_double), ("split", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class BatchStats(ctypes.Structure):
    _fields_ = [("primes", ctypes.c_uint64), ("prime_sum", ctypes.c_uint64),
                ("raw_hits", ctypes.c_uint64), ("factors", ctypes.c_uint64),
                ("steps", ctypes.c_uint64), ("waves", ctypes.c_uint32),
                ("chunk", ctypes.c_uint32), ("unroll", ctypes.c_uint32),
                ("primes_per_lane", ctypes.c_uint32), ("total_ms", ctypes.c_double),
                ("filter_ms", ctypes.c_double), ("sieve_ms", ctypes.c_double),
                ("walk_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class ServerConfig(ctypes.Structure):
    _fields_ = [("factor_bytes", ctypes.c_uint64), ("max_jobs", ctypes.c_uint32),
                ("wave_segments", ctypes.c_uint32), ("wave_work", ctypes.c_uint64)]


class JobResult(ctypes.Structure):
    _fields_ = [("primes", ctypes.c_uint64), ("prime_sum", ctypes.c_uint64),
                ("factors", ctypes.c_uint64), ("latency_ms", ctypes.c_double),
                ("status", ctypes.c_int32), ("pad", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("refused", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("queued", ctypes.c_uint64),
                ("running", ctypes.c_uint64), ("reserved_bytes", ctypes.c_uint64),
                ("primes", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("waves", ctypes.c_uint64), ("chunk", ctypes.c_uint32),
                ("unroll", ctypes.c_uint32), ("busy_ms", ctypes.c_double),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


PPS_JOB_QUEUED, PPS_JOB_RUNNING, PPS_JOB_DONE, PPS_JOB_FAILED = 0, 1, 2, 3
PPS_ERR_FOPEN = -108
PPS_ERR_SCANF = -140


class Checkpoint(ctypes.Structure):
    _fields_ = [("pmin", ctypes.c_uint64), ("p", ctypes.c_uint64), ("count", ctypes.c_uint64),
                ("sum", ctypes.c_uint64), ("nmin", ctypes.c_uint32), ("nmax", ctypes.c_uint32),
                ("factor_count", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


def checkpoint_format(c: Checkpoint, lib=None) -> str:
    """The reference's checkpoint file text (main.c:304-326, pps/app.c:1348-1352)."""
    lib = lib or load()
    buf = ctypes.create_string_buffer(512)
    n = lib.pps_checkpoint_format(ctypes.byref(c), buf, len(buf))
    if n < 0:
        _check(lib, n)
    return buf.value.decode()


def checkpoint_parse(text: str, jp: "JobParams", lib=None) -> Checkpoint:
    lib = lib or load()
    c = Checkpoint()
    _check(lib, lib.pps_checkpoint_parse(text.encode(), ctypes.byref(jp), ctypes.byref(c)))
    return c


class InputInfo(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int32), ("sign", ctypes.c_int32),
                ("records", ctypes.c_uint64), ("k0", ctypes.c_uint64), ("k1", ctypes.c_uint64),
                ("n0", ctypes.c_uint32), ("n1", ctypes.c_uint32)]


class InputFile:
    """An input sieve file (pps_input_read).  `spec` is the job as stated,
    completed from the file where a k or n bound was not given."""

    def __init__(self, path, pmin=0, pmax=0, kmin=0, kmax=0, nmin=0, nmax=0, sign=1, kstep=0,
                 koffset=0, qmax=0, lib=None):
        self.lib = lib or load()
        spec = JobSpec(pmin, pmax, kmin, kmax, nmin, nmax, sign, kstep, koffset, qmax)
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.pps_input_read(str(path).encode(), ctypes.byref(spec),
                                                 ctypes.byref(h)))
        self.h = h
        self.spec = {f: getattr(spec, f) for f, _ in JobSpec._fields_}

    def info(self) -> InputInfo:
        info = InputInfo()
        _check(self.lib, self.lib.pps_input_get_info(self.h, ctypes.byref(info)))
        return info

    def close(self) -> None:
        if self.h:
            self.lib.pps_input_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


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
        "pps_debug_fail_allocs": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
        "pps_debug_limits": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint32]),
        "pps_normalize": (ctypes.c_int, [P(JobSpec), P(JobParams)]),
        "pps_engine_create": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_void_p)]),
        "pps_engine_destroy": (None, [ctypes.c_void_p]),
        "pps_engine_device_bytes": (ctypes.c_uint64, [ctypes.c_void_p]),
        "pps_engine_set_batch_span": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
        "pps_engine_set_variant": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
        "pps_engine_set_split": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
        "pps_engine_set_batch_walk": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
        "pps_walk_variant_name": (ctypes.c_char_p, [ctypes.c_int]),
        "pps_engine_set_wave_segments": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
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
        "pps_run_batch": (ctypes.c_int, [ctypes.c_void_p, P(JobParams), ctypes.c_size_t,
                                         ctypes.c_void_p, ctypes.c_size_t, szp, szp,
                                         P(BatchStats)]),
        "pps_batch_job_primes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, u64p, u64p]),
        "pps_server_create": (ctypes.c_int, [ctypes.c_int, P(ServerConfig), P(ctypes.c_void_p)]),
        "pps_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
        "pps_job_submit": (ctypes.c_int, [ctypes.c_void_p, P(JobParams), u64p]),
        "pps_job_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, P(ctypes.c_int)]),
        "pps_job_cancel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
        "pps_job_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double,
                                        ctypes.c_void_p, ctypes.c_size_t, szp, P(JobResult)]),
        "pps_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, P(ServerStats)]),
        "pps_input_read": (ctypes.c_int, [ctypes.c_char_p, P(JobSpec), P(ctypes.c_void_p)]),
        "pps_input_get_info": (ctypes.c_int, [ctypes.c_void_p, P(InputInfo)]),
        "pps_input_free": (None, [ctypes.c_void_p]),
        "pps_engine_set_input": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
        "pps_checkpoint_format": (ctypes.c_int, [P(Checkpoint), ctypes.c_char_p, ctypes.c_size_t]),
        "pps_checkpoint_parse": (ctypes.c_int, [ctypes.c_char_p, P(JobParams), P(Checkpoint)]),
        "pps_job_checkpoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                              ctypes.c_size_t, szp, P(Checkpoint)]),
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


def walk_variant_name(v: int, lib=None) -> str:
    """The walk variant's short description (pps_walk_variant_name)."""
    return (lib or load()).pps_walk_variant_name(v).decode()


def walk_kernel_name(v: int, lib=None) -> str:
    """The CUDA kernel that runs walk variant v."""
    name = walk_variant_name(v, lib)
    if name.startswith("queue2"):
        return "k_walk32q2"
    if name.startswith(("queue", "twin")):
        return "k_walk32q"
    return "k_walk"


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

    def set_wave_segments(self, segments: int) -> None:
        """Segments per wave of the batched form (before its first use)."""
        _check(self.lib, self.lib.pps_engine_set_wave_segments(self.h, segments))

    def set_batch_walk(self, unroll: int, primes_per_lane: int) -> None:
        """Force the batched walk kernel (8 or 16, 1 or 2); (0, 0): tuned."""
        _check(self.lib, self.lib.pps_engine_set_batch_walk(self.h, unroll, primes_per_lane))

    def set_split(self, t: int) -> None:
        """Force the threads per prime of the queued walks (1, 2, 4, 8; 0: tuned)."""
        _check(self.lib, self.lib.pps_engine_set_split(self.h, t))

    def set_input(self, inp: "InputFile | None") -> None:
        """Use an input sieve file as the output rule (None: the small-prime filter)."""
        self._input = inp  # keep it alive while the engine uses it
        _check(self.lib, self.lib.pps_engine_set_input(self.h, inp.h if inp else None))

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

    def run_batch(self, jobs: list, cap: int = 1 << 18):
        """Batched persistent form: returns (list of per-job factor arrays, BatchStats)."""
        arr = (JobParams * max(len(jobs), 1))(*jobs)
        offs = (ctypes.c_size_t * (len(jobs) + 1))()
        while True:
            out = np.zeros(cap, dtype=FACTOR_DTYPE)
            n = ctypes.c_size_t()
            st = BatchStats()
            rc = self.lib.pps_run_batch(self.h, arr, len(jobs), out.ctypes.data_as(ctypes.c_void_p),
                                        cap, ctypes.byref(n), offs, ctypes.byref(st))
            if rc == PPS_ERR_OVERFLOW and n.value > cap:
                cap = n.value
                continue
            _check(self.lib, rc)
            per = [out[offs[j]:offs[j + 1]].copy() for j in range(len(jobs))]
            return per, st

    def batch_job_primes(self, njobs: int):
        pr = np.zeros(max(njobs, 1), dtype=np.uint64)
        sm = np.zeros(max(njobs, 1), dtype=np.uint64)
        _check(self.lib, self.lib.pps_batch_job_primes(
            self.h, njobs, pr.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            sm.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        return pr[:njobs], sm[:njobs]


def normalize_or_repair(spec: dict, lib=None):
    """Normalise like the reference; where the reference would refuse a job,
    repair it the way its own message suggests and record the repair:
      pmin <= 2^32              -> pmin = 2^32 + 1 (pps/appcu.cu:236-239)
      2^(64-nstep) > pmin       -> double pmin until the rule holds
                                   (the "will work by the time pmin ==" loop,
                                   pps/appcu.cu:163-176)
    The p width is kept.  Returns (JobParams, list of repair strings)."""
    spec = dict(spec)
    repairs = []
    width = spec["pmax"] - spec["pmin"]
    for _ in range(80):
        try:
            return normalize(**spec, lib=lib), repairs
        except PPSError as e:
            msg = str(e)
            if "<= 2^32" in msg:
                spec["pmin"] = (1 << 32) + 1
            elif "pmin is not large enough" in msg:
                spec["pmin"] *= 2
            else:
                raise
            spec["pmax"] = spec["pmin"] + width
            repairs.append(f"pmin->{spec['pmin']}")
    raise PPSError(PPS_ERR_INVALID_PARAM, f"could not repair {spec}")


def mixed_jobs(seed: int = 1, count: int = 512, scale_p: float = 1.0, scale_n: float = 1.0,
               lib=None):
    """The mixed-job workload: `count` jobs drawn from `seed`.  Side +/- uniform;
    kmin odd uniform in [3, 5000]; k width log-uniform in [1e2, 1e4]; nmin uniform
    in [1e3, 1e6]; n width log-uniform in [1e2, 1e6]; pmin log-uniform in
    [1e10, 2^61]; p width log-uniform in [1e7, 1e9] (p > kmax always holds).
    scale_p / scale_n shrink the p and n widths for quick tests.  Returns
    (list of JobParams, list of (spec, repairs))."""
    rng = np.random.default_rng(seed)
    jobs, meta = [], []
    for _ in range(count):
        sign = 1 if rng.integers(0, 2) else -1
        kmin = int(rng.integers(1, 2500)) * 2 + 1
        kw = int(10 ** rng.uniform(2, 4))
        nmin = int(rng.integers(1000, 1000001))
        nw = max(50, int(10 ** rng.uniform(2, 6) * scale_n))
        pmin = int(10 ** rng.uniform(10, np.log10(2.0 ** 61)))
        pw = max(1000, int(10 ** rng.uniform(7, 9) * scale_p))
        spec = dict(pmin=pmin, pmax=pmin + pw, kmin=kmin, kmax=kmin + kw, nmin=nmin, nmax=nmin + nw,
                    sign=sign)
        jp, repairs = normalize_or_repair(spec, lib=lib)
        jobs.append(jp)
        meta.append((spec, repairs))
    return jobs, meta


class Server:
    """The serving loop (pps_server_*): submit normalised jobs, wait for each
    job's sorted factor list."""

    def __init__(self, device: int = 0, factor_bytes: int = 0, max_jobs: int = 0,
                 wave_segments: int = 0, wave_work: int = 0, lib=None):
        self.lib = lib or load()
        cfg = ServerConfig(factor_bytes, max_jobs, wave_segments, int(wave_work))
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.pps_server_create(device, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            self.lib.pps_server_destroy(self.h)
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

    def submit(self, jp: JobParams) -> int:
        jid = ctypes.c_uint64()
        _check(self.lib, self.lib.pps_job_submit(self.h, ctypes.byref(jp), ctypes.byref(jid)))
        return jid.value

    def cancel(self, jid: int) -> None:
        _check(self.lib, self.lib.pps_job_cancel(self.h, jid))

    def poll(self, jid: int) -> int:
        st = ctypes.c_int()
        _check(self.lib, self.lib.pps_job_poll(self.h, jid, ctypes.byref(st)))
        return st.value

    def wait(self, jid: int, timeout: float = -1.0) -> tuple[np.ndarray, JobResult]:
        """Block until job `jid` is done (or `timeout` seconds); returns its
        factors (FACTOR_DTYPE, sorted by p, k, n) and its JobResult."""
        n = ctypes.c_size_t()
        res = JobResult()
        _check(self.lib, self.lib.pps_job_wait(self.h, jid, timeout, None, 0, ctypes.byref(n),
                                               ctypes.byref(res)))
        out = np.zeros(max(n.value, 1), dtype=FACTOR_DTYPE)
        _check(self.lib, self.lib.pps_job_wait(self.h, jid, 0.0, out.ctypes.data_as(ctypes.c_void_p),
                                               out.size, ctypes.byref(n), ctypes.byref(res)))
        return out[: n.value], res

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(self.lib, self.lib.pps_server_get_stats(self.h, ctypes.byref(st)))
        return st

    def checkpoint(self, jid: int) -> tuple[np.ndarray, Checkpoint]:
        """A running job's drained boundary and the factors found below it."""
        c = Checkpoint()
        n = ctypes.c_size_t()
        while True:
            _check(self.lib, self.lib.pps_job_checkpoint(self.h, jid, None, 0, ctypes.byref(n),
                                                         ctypes.byref(c)))
            out = np.zeros(max(n.value, 1) + 64, dtype=FACTOR_DTYPE)
            rc = self.lib.pps_job_checkpoint(self.h, jid, out.ctypes.data_as(ctypes.c_void_p), out.size,
                                             ctypes.byref(n), ctypes.byref(c))
            if rc == PPS_ERR_OVERFLOW:
                continue  # more factors arrived between the two calls
            _check(self.lib, rc)
            return out[: n.value], c
