"""Generate the golden fixtures in tests/golden/ by running the REFERENCE itself.

    make -C oracle refsrc CHECKOUT=<reference checkout>   # stages its C sources
    make -C oracle ref                      # builds oracle/_ref/ from them
    python tests/golden/make_golden.py      # (re)writes tests/golden/ref_cases.json, kat49.json

Needs the reference only through the binaries that `make -C oracle ref`
compiled into oracle/_ref/ (the "files" step also reads the reference's shipped
golden lists, from the checkout named by PPS_REFERENCE):
  ppsieve_ref        the reference's main.c/sieve.c/pps/app.c/pps/factor_proth.c with
                     the CPU stand-in for pps/appcu.h (every subsection flagged);
  tpsieve_ref        its twin build (-DSEARCH_TWIN; steps "twin" and "twin_input");
  ppsieve_ref_fixed  the same with the 64-bit fix at pps/app.c:1087 (used where
                     nstep >= 48, where the unfixed re-walk misses factors).
Each case records the command line, the sorted factor lines and the reference's
own prime fingerprint (count=, sum= from main.c:1232).  The fixtures are small
text; the GPU machine never needs the reference.

kat49.json holds planted factors for nstep >= 48 (p in [9999*2^48, 2^62)): p is a
prime factor of k*2^n-1 or k*2^n+1 for small n found by factoring with sympy;
each is then confirmed by running both reference binaries on a one-prime range.
"""
from __future__ import annotations

import json
import os
import random
import re
import subprocess
import sys
import tempfile
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_DIR = ROOT / "oracle" / "_ref"
REF_BIN = REF_DIR / "ppsieve_ref"
REF_FIXED = REF_DIR / "ppsieve_ref_fixed"

FP_RE = re.compile(r"count=(\d+),sum=0x([0-9a-f]+)")


def run_ref(args: list[str], fixed: bool = False, threads: int = 2) -> dict:
    binary = REF_FIXED if fixed else REF_BIN
    with tempfile.TemporaryDirectory() as td:
        cmd = [str(binary), *args, f"-t{threads}", "-m8192", "-c1000000", "-r1000000", "-q",
               "-fout.txt"]
        t0 = time.time()
        r = subprocess.run(cmd, cwd=td, capture_output=True, text=True)
        dt = time.time() - t0
        out = Path(td, "out.txt")
        lines = [l.strip() for l in out.read_text().splitlines() if "|" in l] if out.exists() else []
    m = FP_RE.search(r.stderr)
    res = {"args": args, "binary": binary.name, "rc": r.returncode, "seconds": round(dt, 2),
           "lines": sorted(lines), "unique": len(set(lines)), "total": len(lines)}
    if m:
        res["count"] = int(m.group(1))
        res["sum"] = "0x" + m.group(2)
    if r.returncode != 0:
        res["stderr_tail"] = r.stderr[-400:]
    return res


def fixed_cases() -> list[tuple[str, list[str], bool]]:
    c = []
    c.append(("small_proth_full", ["-p1e12", "-P1000200000000", "-k1201", "-K9999", "-n2000", "-N3000"], False))
    c.append(("many_n_test", ["-p42070e9", "-P42070050e6", "-k1201", "-K9999", "-N2000000"], False))
    base = 42 * 10**12
    for i, off in enumerate([0, 25 * 10**9, 50 * 10**9, 75 * 10**9, 10**11 - 2 * 10**6]):
        lo = base + off
        c.append((f"large_n_slice{i}", [f"-p{lo}", f"-P{lo + 2 * 10**6}", "-k1201", "-K9999",
                                    "-n2000000", "-N3000000"], False))
    lo3 = (1 << 62) - (1 << 34)
    c.append(("riesel62_slice_lo", [f"-p{lo3}", f"-P{lo3 + 10**7}", "-k3", "-K9999", "-n100000",
                              "-N1000000", "-R"], True))
    c.append(("riesel62_slice_hi", [f"-p{(1 << 62) - 10**7}", f"-P{1 << 62}", "-k3", "-K9999",
                              "-n100000", "-N1000000", "-R"], True))
    # Riesel, small p, many factors
    c.append(("riesel_small", ["-p1e12", "-P1000050000000", "-k1201", "-K9999", "-n2000",
                               "-N3000", "-R"], False))
    # kstep / koffset generality (-M -s), pps/app.c:595-604
    c.append(("kstep6_off3", ["-p1e12", "-P1000050000000", "-k3", "-K9999", "-n2000", "-N4000",
                              "-M6", "-s3"], False))
    # pseudo-prime mode: sieve only with q < 1000 (main.c:971-972 -Q)
    c.append(("qmax_1000", ["-p1e12", "-P1000001000000", "-k1201", "-K9999", "-n2000",
                            "-N3000", "-Q1000"], False))
    # rejected by the reference: auto nmin = 62 < 64 (pps/app.c:683-694, pps/appcu.cu:195)
    c.append(("kround_nauto", ["-p5e11", "-P500020000000", "-k1200", "-K10000", "-N3000"], False))
    # rejected: nstep clamped to nmax-nmin+1 = 11 makes 2^(64-11) > pmin (pps/appcu.cu:160-176)
    c.append(("nstep_clamp", ["-p1e12", "-P1000100000000", "-k1201", "-K9999", "-n2000",
                              "-N2010"], False))
    # even kmin/kmax round to kstep*b+koffset (pps/app.c:705-708)
    c.append(("kround", ["-p1e12", "-P1000050000000", "-k1200", "-K10000", "-n2000", "-N3000"],
              False))
    # nmin from 2*lg2(pmin)-lg2(kmax)-1 (pps/app.c:683-694): 72 here
    c.append(("nmin_auto", ["-p1e13", "-P10000020000000", "-k1201", "-K9999", "-N5000"], False))
    # nstep clamped to nmax-nmin+1 = 10 and still valid at this pmin
    c.append(("nstep_clamp_ok", ["-p2000000000000000000", "-P2000000000010000000", "-k3", "-K9999",
                                 "-n1000", "-N1009"], False))
    # kmin == kmax
    c.append(("single_k", ["-p1e12", "-P1000500000000", "-k9475", "-K9475", "-n2000",
                           "-N9000"], False))
    return c


def random_jobs(seed: int = 20240501, count: int = 40) -> list[tuple[str, list[str], bool]]:
    """Small seeded jobs with the mixed-job distribution's shape (sides, k and n
    widths, p log-uniform), shrunk so the reference finishes each in seconds."""
    rng = random.Random(seed)
    jobs = []
    while len(jobs) < count:
        side = rng.choice([1, -1])
        kmin = rng.randrange(3, 5001) | 1
        kw = int(10 ** rng.uniform(2, 4))
        kmax = kmin + kw
        nmin = rng.randrange(1000, 200000)
        nw = int(10 ** rng.uniform(2, 4.3))
        nmax = nmin + nw
        if len(jobs) % 3 == 2:
            pmin = int(10 ** rng.uniform(14, 18.3))
            pw = int(10 ** rng.uniform(5, 6.3))
        else:
            pmin = int(10 ** rng.uniform(11.8, 14))
            pw = int(10 ** rng.uniform(6, 6.7))
            kw = int(10 ** rng.uniform(3, 4))
            kmax = kmin + kw
            nw = int(10 ** rng.uniform(3.5, 4.5))
            nmax = nmin + nw
        # valid only if the reference's rules accept it (pps/appcu.cu:163)
        ks = (kmax // 2) * 2 + 1
        nstep = 1
        while (ks << nstep) < pmin:
            nstep += 1
        nstep = min(nstep, nmax - nmin + 1)
        if (1 << (64 - nstep)) > pmin or pmin <= (1 << 32):
            continue
        args = [f"-p{pmin}", f"-P{pmin + pw}", f"-k{kmin}", f"-K{kmax}", f"-n{nmin}", f"-N{nmax}"]
        if side < 0:
            args.append("-R")
        jobs.append((f"rand{len(jobs):02d}", args, nstep >= 48))
    return jobs


def planted_kat49(max_found: int = 8, seed: int = 7) -> list[dict]:
    import sympy

    lo, hi = 9999 << 48, 1 << 62
    rng = random.Random(seed)
    found = []
    tried = 0
    while len(found) < max_found and tried < 20000:
        tried += 1
        n = rng.randrange(64, 84)
        k = rng.randrange(3, 10000) | 1
        c = rng.choice([1, -1])
        N = k * (1 << n) + c
        f = sympy.factorint(N, limit=1 << 22)
        if min(f) < 32768:
            continue  # the output rule would drop the line (pps/app.c:171-179)
        for q, e in f.items():
            if lo <= q < hi and sympy.isprime(q):
                found.append({"p": int(q), "k": k, "n": n, "c": c})
        if tried % 500 == 0:
            print(f"  kat49: tried {tried}, found {len(found)}", flush=True)
    return found


INPUTS = HERE / "inputs"
SMALL_Q = (3, 5, 7, 11, 13, 17, 19, 23, 29)


def _survivors(kmin: int, kmax: int, nmin: int, nmax: int, c: int) -> list[tuple[int, int]]:
    """(k, n) with k odd, nmin <= n <= nmax, k*2^n+c free of the primes below 30:
    a stand-in for the output of a sieving program such as NewPGen."""
    out = []
    for k in range(kmin | 1, kmax + 1, 2):
        for n in range(nmin, nmax + 1):
            if all((k * pow(2, n, q) + c) % q for q in SMALL_Q):
                out.append((k, n))
    return out


def write_newpgen(path: Path, pairs, c: int) -> None:
    """NewPGen format as pps/app.c:221-230 reads it: "p0:P:x:2:c" then "k n" lines."""
    lines = [f"30:P:1:2:{c}"] + [f"{k} {n}" for k, n in sorted(pairs)]
    path.write_text("\n".join(lines) + "\n")


def write_abcd(path: Path, pairs, c: int) -> None:
    """ABCD format as pps/app.c:213-218 and 405-500 read it: per k a header
    "ABCD k*2^$a+1 [n0]" then one n delta per line."""
    by_k: dict[int, list[int]] = {}
    for k, n in sorted(pairs):
        by_k.setdefault(k, []).append(n)
    out = []
    sign = "+" if c > 0 else "-"
    for k, ns in by_k.items():
        out.append(f"ABCD {k}*2^$a{sign}1 [{ns[0]}] // sieved to 30")
        out += [str(b - a) for a, b in zip(ns, ns[1:])]
    path.write_text("\n".join(out) + "\n")


def _twin_survivors(kmin: int, kmax: int, nmin: int, nmax: int) -> list[tuple[int, int]]:
    """(k, n) with k == 3 (mod 6), nmin <= n <= nmax, both k*2^n+1 and k*2^n-1
    free of the primes below 30: a stand-in for a twin sieve's output."""
    out = []
    for k in range(kmin + (3 - kmin) % 6, kmax + 1, 6):
        for n in range(nmin, nmax + 1):
            if all((k * pow(2, n, q) + 1) % q and (k * pow(2, n, q) - 1) % q for q in SMALL_Q):
                out.append((k, n))
    return out


def write_twin_newpgen(path: Path, pairs) -> None:
    """The twin build's NewPGen format (pps/app.c:214-215, 360-365): "p0:T:x:2:3"
    then "k n" lines."""
    lines = ["30:T:1:2:3"] + [f"{k} {n}" for k, n in sorted(pairs)]
    path.write_text("\n".join(lines) + "\n")


def write_twin_abcd(path: Path, pairs) -> None:
    """The twin build's ABCD format (pps/app.c:212-213, 429-500): per n a header
    "ABCD (6*$a+3)*2^n+1 & (6*$a+3)*2^n-1 [a0]" with k = 6a + 3, then one a
    delta per line."""
    by_n: dict[int, list[int]] = {}
    for k, n in sorted(pairs, key=lambda t: (t[1], t[0])):
        by_n.setdefault(n, []).append((k - 3) // 6)
    out = []
    for n, a in sorted(by_n.items()):
        out.append(f"ABCD (6*$a+3)*2^{n}+1 & (6*$a+3)*2^{n}-1 [{a[0]}] // sieved to 30")
        out += [str(y - x) for x, y in zip(a, a[1:])]
    path.write_text("\n".join(out) + "\n")


def make_twin_input_cases() -> None:
    """Synthetic twin sieve files in both of the twin build's formats, and the
    reference's twin build's own output when given each with -i."""
    INPUTS.mkdir(exist_ok=True)
    pairs = _twin_survivors(3, 99, 1000, 2999)
    write_twin_newpgen(INPUTS / "twin_newpgen.txt", pairs)
    write_twin_abcd(INPUTS / "twin_abcd.txt", pairs)
    print("twin input pairs:", len(pairs), flush=True)
    lo = 5 * 10**10
    rng = [f"-p{lo}", f"-P{lo + 10**9}"]
    cases = [
        ("twin_in_newpgen", "twin_newpgen.txt", rng),
        ("twin_in_abcd", "twin_abcd.txt", rng),
        # a partial override: kmax given, the rest from the file
        ("twin_in_abcd_kmax", "twin_abcd.txt", [*rng, "-K51"]),
        # all of k/n given: the file is read as ABCD without a scan (pps/app.c:97);
        # the ranges cover the file's, so the reference's bitmap holds every entry
        ("twin_in_abcd_given", "twin_abcd.txt", [*rng, "-k3", "-K99", "-n1000", "-N3000"]),
        # and a NewPGen file is then an invalid header (ERR_SCANF)
        ("twin_in_newpgen_given", "twin_newpgen.txt", [*rng, "-k3", "-K99", "-n1000", "-N3000"]),
    ]
    binary = REF_DIR / "tpsieve_ref"

    def one(case):
        name, f, args = case
        with tempfile.TemporaryDirectory() as td:
            cmd = [str(binary), *args, f"-i{INPUTS / f}", "-t2", "-m8192", "-c1000000", "-r1000000", "-q",
                   "-fout.txt"]
            r = subprocess.run(cmd, cwd=td, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True,
                               timeout=1200)
            out = Path(td, "out.txt")
            lines = [l.strip() for l in out.read_text().splitlines() if "|" in l] if out.exists() else []
        m = FP_RE.search(r.stderr)
        res = {"args": args, "input": f, "binary": binary.name, "rc": r.returncode, "lines": sorted(lines),
               "unique": len(set(lines)), "total": len(lines)}
        if m:
            res["count"] = int(m.group(1))
            res["sum"] = "0x" + m.group(2)
        print(f"{name}: {len(lines)} lines rc={r.returncode}", flush=True)
        return name, res

    with ThreadPoolExecutor(max_workers=2) as ex:
        out = dict(ex.map(one, cases))
    (HERE / "twin_input_cases.json").write_text(json.dumps(out, indent=1, sort_keys=True))


def make_input_cases() -> None:
    """Synthetic sieve files in both formats and both signs, and the reference's
    own output when given each with -i (bitmap output rule, pps/app.c:180-183)."""
    INPUTS.mkdir(exist_ok=True)
    files = {}
    for c in (1, -1):
        pairs = _survivors(3, 99, 1000, 1999, c)
        tag = "proth" if c > 0 else "riesel"
        write_newpgen(INPUTS / f"newpgen_{tag}.txt", pairs, c)
        write_abcd(INPUTS / f"abcd_{tag}.txt", pairs, c)
        files[tag] = len(pairs)
    print("input files:", files, flush=True)
    lo = 5 * 10**10
    cases = []
    for fmt in ("newpgen", "abcd"):
        for tag in ("proth", "riesel"):
            f = f"{fmt}_{tag}.txt"
            # ranges from the file (the reference's scan_input_file, pps/app.c:190-347)
            cases.append((f"in_{fmt}_{tag}", f, [f"-p{lo}", f"-P{lo + 25 * 10**8}"]))
    # k/n all given: no scan, so no format detection either: the file is read as
    # ABCD (pps/app.c:97), and a NewPGen file is refused (ERR_SCANF, exit 116)
    cases.append(("in_newpgen_proth_given", "newpgen_proth.txt",
                  [f"-p{lo}", f"-P{lo + 25 * 10**8}", "-k11", "-K61", "-n1200", "-N1800"]))
    # ABCD against given ranges, -R by option.  The k range covers the file's:
    # pps/app.c:440-447 does not check k, so a k below kmin writes outside the
    # reference's bitmap (it crashed on that here), and headers' n are unchecked
    # above nmax; both are left out of the fixtures.
    cases.append(("in_abcd_riesel_given", "abcd_riesel.txt",
                  [f"-p{lo}", f"-P{lo + 25 * 10**8}", "-k3", "-K99", "-n1200", "-N1800", "-R"]))
    # a partial override: kmax given, the rest from the file
    cases.append(("in_abcd_proth_kmax", "abcd_proth.txt", [f"-p{lo}", f"-P{lo + 25 * 10**8}", "-K51"]))

    def one(case):
        name, f, args = case
        r = run_ref([*args, f"-i{INPUTS / f}"], threads=2)
        r["args"] = args
        r["input"] = f
        print(f"{name}: {r['total']} lines rc={r['rc']}", flush=True)
        return name, r

    with ThreadPoolExecutor(max_workers=4) as ex:
        out = dict(ex.map(one, cases))
    (HERE / "input_cases.json").write_text(json.dumps(out, indent=1, sort_keys=True))


def main() -> None:
    if not REF_BIN.exists() or not REF_FIXED.exists():
        sys.exit("build the reference first: make -C oracle ref")
    which = sys.argv[1:] or ["cases", "kat"]
    only = set(which[1:]) if which and which[0] == "cases" else set()
    if "cases" in which:
        cases = fixed_cases() + random_jobs()
        if only:
            cases = [c for c in cases if c[0] in only or (c[0].startswith("rand") and "rand" in only)]
        out_json = HERE / "ref_cases.json"
        results = json.loads(out_json.read_text()) if (only and out_json.exists()) else {}
        if only:
            for k in list(results):
                if k.startswith("rand") and "rand" in only:
                    del results[k]
        heavy = {"many_n_test", "small_proth_full", "riesel62_slice_lo", "riesel62_slice_hi"}

        def one(case):
            name, args, fixed = case
            t = 8 if name in heavy else 2
            r = run_ref(args, fixed=fixed, threads=t)
            print(f"{name}: {r['total']} lines in {r['seconds']} s rc={r['rc']}", flush=True)
            return name, r

        light = [c for c in cases if c[0] not in heavy]
        with ThreadPoolExecutor(max_workers=3) as ex:
            for name, r in ex.map(one, light):
                results[name] = r
        for c in cases:
            if c[0] in heavy:
                name, r = one(c)
                results[name] = r
        if not only:
            # as-is reference on the nstep>=48 slice too, to record its divergence
            lo3 = (1 << 62) - (1 << 34)
            r = run_ref([f"-p{lo3}", f"-P{lo3 + 10**7}", "-k3", "-K9999", "-n100000", "-N1000000",
                         "-R"], fixed=False, threads=8)
            results["riesel62_slice_lo_asis"] = r
        out_json.write_text(json.dumps(results, indent=1, sort_keys=True))
    if "files" in which:
        # The reference's own golden lists, sorted: pps/oldsort.txt (the older,
        # unfiltered many_n_test.sh output) and pps/pps_test_ok.txt; and the
        # many_n_test.sh range as the current reference prints it (from its run).
        if not os.environ.get("PPS_REFERENCE"):
            sys.exit("the files step reads pps/oldsort.txt and pps/pps_test_ok.txt: "
                     "set PPS_REFERENCE=<reference checkout>")
        ref_root = Path(os.environ["PPS_REFERENCE"])
        for src, dst in (("pps/oldsort.txt", "oldsort_144.txt"),
                         ("pps/pps_test_ok.txt", "pps_test_ok_15.txt")):
            lines = sorted(l.strip() for l in (ref_root / src).read_text().splitlines()
                           if "|" in l)
            (HERE / dst).write_text("\n".join(lines) + "\n")
        cases = json.loads((HERE / "ref_cases.json").read_text())
        (HERE / "many_n_test_39.txt").write_text("\n".join(cases["many_n_test"]["lines"]) + "\n")
    if "twin" in which:
        # the reference's twin build (tpsieve_ref: -DSEARCH_TWIN, both sides per walk,
        # k == 3 mod 6 unless -M/-s say otherwise)
        rng = random.Random(99)
        cases = [
            ("twin_small", ["-p1e12", "-P1000050000000", "-k1201", "-K9999", "-n2000", "-N3000"]),
            ("twin_all_odd_k", ["-p1e12", "-P1000020000000", "-k3", "-K9999", "-n2000", "-N3000",
                                "-M2", "-s1"]),
            ("twin_large_n_slice", [f"-p{42 * 10**12}", f"-P{42 * 10**12 + 2 * 10**6}", "-k1201",
                               "-K9999", "-n2000000", "-N3000000"]),
            ("twin_nstep32", [f"-p{2**40}", f"-P{2**40 + 10**7}", "-k3", "-K999", "-n100000",
                              "-N101000", "-M2", "-s1"]),
            ("twin_wide_n", ["-p1e12", "-P1000020000000", "-k3", "-K9999", "-n1000", "-N100000",
                             "-M2", "-s1"]),
            ("twin_wide_n3", ["-p2e12", "-P2000030000000", "-k1201", "-K9999", "-n1000",
                              "-N200000"]),
        ]
        for i in range(10):
            pmin = int(10 ** rng.uniform(11.5, 15.5))
            kmin = rng.randrange(3, 3000)
            n0 = rng.randrange(200, 200000)
            cases.append((f"twin_rand{i:02d}", [f"-p{pmin}", f"-P{pmin + rng.randrange(10**6, 10**7)}",
                                                f"-k{kmin}", f"-K{kmin + rng.randrange(100, 9000)}",
                                                f"-n{n0}", f"-N{n0 + rng.randrange(100, 20000)}"]))
        binary = REF_DIR / "tpsieve_ref"

        def one_twin(case):
            name, args = case
            with tempfile.TemporaryDirectory() as td:
                cmd = [str(binary), *args, "-t2", "-m8192", "-c1000000", "-r1000000", "-q", "-fout.txt"]
                r = subprocess.run(cmd, cwd=td, capture_output=True, text=True)
                out = Path(td, "out.txt")
                lines = [l.strip() for l in out.read_text().splitlines() if "|" in l] if out.exists() else []
            m = FP_RE.search(r.stderr)
            res = {"args": args, "binary": binary.name, "rc": r.returncode, "lines": sorted(lines),
                   "unique": len(set(lines)), "total": len(lines)}
            if m:
                res["count"] = int(m.group(1))
                res["sum"] = "0x" + m.group(2)
            print(f"{name}: {len(lines)} lines rc={r.returncode}", flush=True)
            return name, res

        with ThreadPoolExecutor(max_workers=4) as ex:
            out = dict(ex.map(one_twin, cases))
        (HERE / "twin_cases.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    if "input" in which:
        make_input_cases()
    if "twin_input" in which:
        make_twin_input_cases()
    if "kat" in which:
        kats = planted_kat49()
        out = []
        for kat in kats:
            p = kat["p"]
            # nmin/nmax around n with nstep = 49: kmax*2^48 < pmin
            nmin, nmax = 64, 160
            args = [f"-p{p}", f"-P{p + 2}", "-k3", "-K9999", f"-n{nmin}", f"-N{nmax}"]
            if kat["c"] < 0:
                args.append("-R")
            rf = run_ref(args, fixed=True, threads=1)
            ra = run_ref(args, fixed=False, threads=1)
            out.append({**kat, "args": args, "fixed_lines": rf["lines"], "asis_lines": ra["lines"]})
            print(f"kat p={p} k={kat['k']} n={kat['n']} c={kat['c']}: fixed {len(rf['lines'])} "
                  f"as-is {len(ra['lines'])}", flush=True)
        (HERE / "kat49.json").write_text(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
