"""Python binding of the CPU oracle (oracle/_build/libppsoracle.so).

ORACLE / TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke()
as the checker and by bench.py's CPU-baseline leg.  The shipped library never
imports it.  The C code it wraps restates the reference's CPU path; see
pps_oracle.h for the file:line map.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libppsoracle.so"
CLI = HERE / "_build" / "pps_oracle"
REF_DIR = HERE / "_ref"

FACTOR_DTYPE = np.dtype([("p", "<u8"), ("k", "<u8"), ("n", "<u4"), ("c", "<i4")])


class Params(ctypes.Structure):
    _fields_ = [("pmin", ctypes.c_uint64), ("pmax", ctypes.c_uint64),
                ("kmin", ctypes.c_uint64), ("kmax", ctypes.c_uint64),
                ("nmin", ctypes.c_uint32), ("nmax", ctypes.c_uint32),
                ("c", ctypes.c_int32), ("kstep", ctypes.c_uint32),
                ("koffset", ctypes.c_uint32), ("qmax", ctypes.c_uint32),
                ("nstep", ctypes.c_uint32), ("pad0", ctypes.c_uint32),
                ("input_keys", ctypes.c_void_p), ("ninput", ctypes.c_uint64),
                ("input_width", ctypes.c_uint64)]
    _INPUT_FIELDS = ("pad0", "input_keys", "ninput", "input_width")

    def as_dict(self) -> dict:
        """The job's parameters (the input-file fields excluded)."""
        return {f: getattr(self, f) for f, _ in self._fields_ if f not in self._INPUT_FIELDS}


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = ctypes.CDLL(str(LIB))
        P = ctypes.POINTER
        lib.ppo_normalize.restype = ctypes.c_int
        lib.ppo_normalize.argtypes = [P(Params), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                      ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_uint32]
        lib.ppo_run.restype = ctypes.c_long
        lib.ppo_run.argtypes = [P(Params), ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                P(ctypes.c_uint64), P(ctypes.c_uint64)]
        lib.ppo_walk_list.restype = ctypes.c_long
        lib.ppo_walk_list.argtypes = [P(Params), P(ctypes.c_uint64), ctypes.c_size_t, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_size_t]
        lib.ppo_walk_prime_raw.restype = ctypes.c_size_t
        lib.ppo_walk_prime_raw.argtypes = [P(Params), ctypes.c_uint64, ctypes.c_void_p,
                                           ctypes.c_size_t]
        lib.ppo_small_factor.restype = ctypes.c_uint32
        lib.ppo_small_factor.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32]
        lib.ppo_small_factor_from.restype = ctypes.c_uint32
        lib.ppo_small_factor_from.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32,
                                              ctypes.c_uint32]
        lib.ppo_test_factor.restype = ctypes.c_int
        lib.ppo_test_factor.argtypes = [P(Params), ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32]
        lib.ppo_is_prime.restype = ctypes.c_int
        lib.ppo_is_prime.argtypes = [ctypes.c_uint64]
        lib.ppo_kpow_mod.restype = ctypes.c_uint64
        lib.ppo_kpow_mod.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64]
        lib.ppo_sieve_fingerprint.restype = ctypes.c_int
        lib.ppo_sieve_fingerprint.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                              ctypes.c_int, P(ctypes.c_uint64), P(ctypes.c_uint64)]
        lib.ppo_verify_factors.restype = ctypes.c_long
        lib.ppo_verify_factors.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
        lib.ppo_sieve_range.restype = ctypes.c_size_t
        lib.ppo_sieve_range.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                        P(ctypes.c_uint64), ctypes.c_size_t]
        _lib = lib
    return _lib


class OracleError(ValueError):
    pass


def normalize(pmin=0, pmax=0, kmin=0, kmax=0, nmin=0, nmax=0, sign=1, kstep=0, koffset=0,
              qmax=0) -> Params:
    lib = load()
    p = Params()
    rc = lib.ppo_normalize(ctypes.byref(p), pmin, pmax, kmin, kmax, nmin, nmax, sign, kstep,
                           koffset, qmax)
    if rc:
        raise OracleError(rc)
    return p


def threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def run(params: Params, nthreads: int | None = None, cap: int = 1 << 16):
    """Whole range on the CPU: (factors ndarray sorted by (p,k,n), count, sum)."""
    lib = load()
    while True:
        out = np.zeros(cap, dtype=FACTOR_DTYPE)
        cnt, s = ctypes.c_uint64(), ctypes.c_uint64()
        n = lib.ppo_run(ctypes.byref(params), nthreads or threads(),
                        out.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(cnt),
                        ctypes.byref(s))
        if n > cap:
            cap = n
            continue
        return out[:n].copy(), cnt.value, s.value


def walk_list(params: Params, primes, nthreads: int | None = None, cap: int = 1 << 16):
    lib = load()
    P = np.ascontiguousarray(primes, dtype=np.uint64)
    while True:
        out = np.zeros(cap, dtype=FACTOR_DTYPE)
        n = lib.ppo_walk_list(ctypes.byref(params), P.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                              len(P), nthreads or threads(), out.ctypes.data_as(ctypes.c_void_p), cap)
        if n > cap:
            cap = n
            continue
        return out[:n].copy()


def raw_candidates(params: Params, primes) -> list[tuple[int, int, int]]:
    """(p, k, n) before the output filter, for every prime in the list."""
    lib = load()
    out = np.zeros(256, dtype=FACTOR_DTYPE)
    res = []
    for p in primes:
        n = lib.ppo_walk_prime_raw(ctypes.byref(params), int(p),
                                   out.ctypes.data_as(ctypes.c_void_p), len(out))
        assert n <= len(out)
        res.extend((int(r["p"]), int(r["k"]), int(r["n"])) for r in out[:n])
    return res


def sieve_range(lo: int, hi: int, qmax: int) -> np.ndarray:
    lib = load()
    n = lib.ppo_sieve_range(lo, hi, qmax, None, 0)
    out = np.zeros(max(n, 1), dtype=np.uint64)
    lib.ppo_sieve_range(lo, hi, qmax, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n)
    return out[:n]


def fingerprint(lo: int, hi: int, qmax: int, nthreads: int | None = None) -> tuple[int, int]:
    """(count, 64-bit wrapping sum) of the primes in [lo, hi) under the sieve
    rule with bound qmax: the reference's count=/sum= line for a whole range."""
    cnt, s = ctypes.c_uint64(), ctypes.c_uint64()
    load().ppo_sieve_fingerprint(lo, hi, qmax, nthreads or threads(), ctypes.byref(cnt), ctypes.byref(s))
    return cnt.value, s.value


BAD_BITS = {1: "p not prime", 2: "p out of range", 4: "k out of range or residue", 8: "n out of range",
            16: "wrong side", 32: "p does not divide k*2^n+c", 64: "output rule"}


def verify_factors(jobs, factors, job_of=None, nthreads: int | None = None):
    """Per-line verification of reported factors (kept as the oracle for every
    run): `jobs` a Params or a list of them, `factors` rows with fields p, k, n,
    c, `job_of` the job index of each row (None: all rows of jobs[0]).
    Returns (failures, bad) with bad[i] the failed-check bits of row i."""
    lib = load()
    if isinstance(jobs, Params):
        jobs = [jobs]
    arr = (Params * len(jobs))(*jobs)
    f = np.zeros(len(factors), dtype=FACTOR_DTYPE)
    for name in ("p", "k", "n", "c"):
        f[name] = factors[name]
    jo = None
    if job_of is not None:
        jo = np.ascontiguousarray(job_of, dtype=np.uint32)
        assert len(jo) == len(f) and (len(jo) == 0 or int(jo.max()) < len(jobs))
    bad = np.zeros(len(f), dtype=np.uint8)
    fails = lib.ppo_verify_factors(ctypes.cast(arr, ctypes.c_void_p),
                                   jo.ctypes.data if jo is not None else None,
                                   f.ctypes.data, len(f), nthreads or threads(), bad.ctypes.data)
    return int(fails), bad


def small_factor(k: int, n: int, c: int, qmin: int = 3) -> int:
    return int(load().ppo_small_factor_from(k, n, c, qmin))


def test_factor(params: Params, k: int, n: int, c: int) -> bool:
    return bool(load().ppo_test_factor(ctypes.byref(params), k, n, c))


def is_prime(x: int) -> bool:
    return bool(load().ppo_is_prime(x))


def kpow_mod(k: int, n: int, c: int, p: int) -> int:
    return int(load().ppo_kpow_mod(k, n, c, p))


def verify_line(p: int, k: int, n: int, c: int) -> bool:
    """Per-line check kept for every run: p prime and p | k*2^n+c."""
    return is_prime(p) and kpow_mod(k, n, c, p) == 0


def tuples(arr) -> list[tuple[int, int, int, int]]:
    return [(int(r["p"]), int(r["k"]), int(r["n"]), int(r["c"])) for r in arr]


def format_line(p: int, k: int, n: int, c: int) -> str:
    return f"{p} | {k}*2^{n}{c:+d}"


def parse_line(line: str) -> tuple[int, int, int, int]:
    left, right = line.split("|")
    p = int(left.strip())
    kpart, rest = right.strip().split("*2^")
    if "+" in rest:
        n, c = rest.split("+")
        return p, int(kpart), int(n), int(c)
    n, c = rest.split("-")
    return p, int(kpart), int(n), -int(c)


# ---------------------------------------------------------------- input files

ERR_SCANF = -140  # pps/app.h:69
TWIN = 2  # sign of a twin job (PPO_TWIN)


class InputFile:
    """A sieve file as the reference reads it (pps/app.c:190-517): NewPGen
    ("p0:P:x:2:c" then "k n" lines) or ABCD ("ABCD k*2^$a+1 [n0]" then n
    deltas).  records: (k, n) in file order; k0..k1, n0..n1 the scan's extents
    (n1 one past the largest n, pps/app.c:319)."""

    def __init__(self, fmt: str, sign: int, records: list[tuple[int, int]]):
        self.format, self.sign, self.records = fmt, sign, records
        ks = [k for k, _ in records]
        ns = [n for _, n in records]
        self.k0, self.k1 = min(ks), max(ks)
        self.n0, self.n1 = min(ns), max(ns) + 1


def read_twin_input(path, detect: bool = True) -> InputFile:
    """The twin build's formats (pps/app.c:208-216 headers, 242-309 scan,
    349-517 read with SEARCH_TWIN): NewPGen "p0:T:x:2:3" then "k n" lines, or
    ABCD "ABCD (6*$a+3)*2^n+1 & (6*$a+3)*2^n-1 [a0]" per n with a deltas, a
    being the k index (k = kstep a + koffset).  ABCD records hold (a, n) and
    format "abcd_twin"; the scan's k extents are indices too (converted in
    input_spec, pps/app.c:325-331)."""
    import re

    text = open(path).read().splitlines()
    hdr = r"\s*ABCD \(6\*\$a\+3\)\*2\^(\d+)\+1 & \(6\*\$a\+3\)\*2\^(\d+)-1 \[(\d+)\]"
    m = re.match(hdr, text[0]) if text else None
    if m and m.group(1) == m.group(2):
        recs, n, a = [], int(m.group(1)), int(m.group(3))
        recs.append((a, n))
        for line in text[1:]:
            h = re.match(hdr, line)
            if h:
                if h.group(1) != h.group(2):
                    break
                n, a = int(h.group(1)), int(h.group(3))
                recs.append((a, n))
                continue
            d = re.match(r"(\d+)", line)
            if not d:
                if line.strip():
                    break
                continue  # blank line
            a += int(d.group(1))
            recs.append((a, n))
        return InputFile("abcd_twin", TWIN, recs)
    if not detect:
        raise OracleError(ERR_SCANF)
    m = re.match(r"\s*(\d+):T:.:2:(.)", text[0]) if text else None
    if not m or m.group(2) != "3":
        raise OracleError(ERR_SCANF)
    recs = []
    for line in text[1:]:
        f = line.split()
        if len(f) < 2:
            break
        recs.append((int(f[0]), int(f[1])))
    if not recs:
        raise OracleError(ERR_SCANF)  # "Invalid line 2"
    return InputFile("newpgen", TWIN, recs)


def read_input(path, detect: bool = True, twin: bool = False) -> InputFile:
    """Format detection and parsing (pps/app.c:208-231 headers, 242-309 scan,
    349-517 read).  The reference detects the format only while scanning (when
    one of kmin, kmax, nmin, nmax is not given); otherwise it reads the file as
    ABCD (pps/app.c:97), and a NewPGen file is an invalid header.  twin: the
    twin build's formats (read_twin_input)."""
    import re

    if twin:
        return read_twin_input(path, detect)
    text = open(path).read().splitlines()
    m = re.match(r"ABCD (\d+)\*2\^\$a([+-])1 \[(\d+)\]", text[0]) if text else None
    if not m and not detect:
        raise OracleError(ERR_SCANF)
    if m:
        recs, k, n = [], int(m.group(1)), int(m.group(3))
        sign = 1 if m.group(2) == "+" else -1
        recs.append((k, n))
        for line in text[1:]:
            h = re.match(r"\s*ABCD (\d+)\*2\^\$a[+-]1 \[(\d+)\]", line)
            if h:
                k, n = int(h.group(1)), int(h.group(2))
                recs.append((k, n))
                continue
            d = re.match(r"(\d+)", line)
            if not d:
                continue  # blank line
            n += int(d.group(1))
            recs.append((k, n))
        return InputFile("abcd", sign, recs)
    m = re.match(r"\s*(\d+):P:.:2:(-?\d+)", text[0]) if text else None
    if not m or int(m.group(2)) not in (1, -1, 255, 257):
        raise OracleError(ERR_SCANF)
    c = int(m.group(2))
    sign = 1 if c in (1, 257) else -1  # (char) of the header's c
    recs = []
    for line in text[1:]:
        f = line.split()
        if len(f) < 2:
            break
        recs.append((int(f[0]), int(f[1])))
    if not recs:
        raise OracleError(ERR_SCANF)  # "Invalid line 2"
    return InputFile("newpgen", sign, recs)


def input_spec(inp: InputFile, spec: dict) -> dict:
    """The scan's effect on the job (pps/app.c:661-663, 335-346): only when one
    of kmin, kmax, nmin, nmax is not given; the file's side is taken then."""
    spec = dict(spec)
    if all(spec.get(f) for f in ("kmin", "kmax", "nmin", "nmax")):
        return spec
    spec["sign"] = inp.sign
    k0, k1 = inp.k0, inp.k1
    if inp.format == "abcd_twin":  # indices to k (pps/app.c:325-331)
        kstep = spec.get("kstep") or 6
        koffset = spec.get("koffset") or 3
        k0, k1 = kstep * k0 + koffset, kstep * k1 + koffset
    spec["kmin"] = max(spec.get("kmin") or 0, k0)
    if not spec.get("kmax") or spec["kmax"] > k1:
        spec["kmax"] = k1
    spec["nmin"] = max(spec.get("nmin") or 0, inp.n0)
    if not spec.get("nmax") or spec["nmax"] > inp.n1:
        spec["nmax"] = inp.n1
    return spec


def input_keys(inp: InputFile, params: Params) -> np.ndarray:
    """The file's bitmap (pps/app.c:726-737, 383-392, 440-478) as sorted keys
    (n - nmin) * width + (k - kmin) / kstep.  NewPGen lines must have
    k == koffset (mod kstep) (pps/app.c:385-389).  Entries whose bit would fall
    outside the reference's bitmap are left out."""
    kstep, koffset = params.kstep, params.koffset
    width = (params.kmax - params.kmin) // kstep + 1
    b0 = (params.kmin - koffset) // kstep
    keys = set()
    for k, n in inp.records:
        if inp.format == "newpgen":
            if k % kstep != koffset:
                raise OracleError(ERR_SCANF)
            if not (params.kmin <= k <= params.kmax):
                continue
            bit = k // kstep - b0
        elif inp.format == "abcd_twin":  # k is the index a (pps/app.c:451, 484)
            if k < b0:
                continue
            bit = k - b0
            if bit >= width:
                continue
        else:
            if k < params.kmin:
                continue
            bit = (k - params.kmin) // kstep
            if bit >= width:
                continue
        if params.nmin <= n <= params.nmax:
            keys.add((n - params.nmin) * width + bit)
    return np.array(sorted(keys), dtype=np.uint64)


def attach_input(params: Params, keys: np.ndarray) -> Params:
    """Use the file as the output rule of `params` (keys stay referenced)."""
    params._keys = keys
    params.input_keys = keys.ctypes.data if len(keys) else None
    params.ninput = len(keys)
    params.input_width = (params.kmax - params.kmin) // params.kstep + 1
    if not len(keys):
        # an empty file set reports nothing: a key no candidate can have
        params._keys = np.array([np.iinfo(np.uint64).max], dtype=np.uint64)
        params.input_keys = params._keys.ctypes.data
        params.ninput = 1
    return params
