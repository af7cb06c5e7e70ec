"""Shared test helpers: parse the reference's option strings into job specs."""
from __future__ import annotations


def parse_num(s: str) -> int:
    """Number syntax of the reference's parse_uint64 (putil.c:86-168)."""
    mult = {"K": 10**3, "M": 10**6, "G": 10**9, "T": 10**12, "P": 10**15,
            "k": 1 << 10, "m": 1 << 20, "g": 1 << 30, "t": 1 << 40, "p": 1 << 50}
    if s[-1] in mult:
        return int(s[:-1], 0) * mult[s[-1]]
    for sep in ("e", "E"):
        if sep in s and not s.lower().startswith("0x"):
            a, b = s.split(sep)
            return int(a, 0) * 10 ** int(b)
    for sep in ("b", "B"):
        if sep in s and not s.lower().startswith("0x"):
            a, b = s.split(sep)
            return int(a, 0) << int(b)
    return int(s, 0)


def args_to_spec(args: list[str]) -> dict:
    spec = dict(pmin=0, pmax=0, kmin=0, kmax=0, nmin=0, nmax=0, sign=1, kstep=0, koffset=0, qmax=0)
    keys = {"p": "pmin", "P": "pmax", "k": "kmin", "K": "kmax", "n": "nmin", "N": "nmax",
            "M": "kstep", "s": "koffset", "Q": "qmax"}
    for a in args:
        assert a.startswith("-")
        o, v = a[1], a[2:]
        if o == "R":
            spec["sign"] = -1
        elif o in keys:
            spec[keys[o]] = parse_num(v)
            if o == "M" and spec["koffset"] >= spec["kstep"]:
                spec["koffset"] = spec["kstep"] // 2
        else:
            raise ValueError(a)
    return spec


def lines_of(tuples) -> list[str]:
    return sorted(f"{p} | {k}*2^{n}{c:+d}" for p, k, n, c in tuples)
