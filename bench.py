"""Benchmark of the PPSieve hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload ("large-n Proth"): odd k in [1201, 9999],
n in [2,000,000, 3,000,000), primes p in [4.2e13, 4.2e13 + 1e11).  One step is
one pass of the hot path over one batch: the device sieve of the next 2^31-wide
slice of that p range (about 6.8e7 primes), the walk of every prime over the
whole n range, and the output filter.  Step i takes slice i, so the timed steps
cover K consecutive slices of the workload's range (47 slices make the whole
range).  Inputs are generated on the device (the slice's primes are 1.1 GB,
larger than the 129 MB L2, so no flush is needed between steps).

value  = primes fully walked per second (whole job, all ranks).
e2e    = the same metric through the drop-in C-ABI call with HOST buffers:
         pps_check_primes() given the slice's primes in pinned host memory
         (read by the walk in place over the host link, inside the timed
         region) and returning the factor list to the host (D2H inside the
         timed region) -- what the reference's check_ns / get_factors_found
         boundary carries.
roofline: the walk kernel is bound by the 32-bit integer multiply pipe; its
         algorithmic work is 3 multiplies per walk step (one 32 n-values advance
         of one prime); the peak is the multiply-pipe throughput measured in this
         run by pps_measure_imad_peak on the same multiply mix.
verify : the checker leg, after every timed leg and not timed: the large-n
         Proth workload (47 slices) and the 62-bit Riesel workload
         (p in [2^62 - 2^34, 2^62), 8 slices) run in full on the GPU; every
         factor the bench reported (the full runs, the timed slices, the
         host-buffer path, the 512-job mix, the served jobs) is verified line by
         line by the oracle on the host cores, and the prime count and sum of
         every full-range slice (and of 16 seeded mixed jobs) are compared with
         the oracle's sieve.
reference_gpu: the reference's own GPU program (its main.c, sieve.c, pps/app.c
         and CUDA kernels built for this GPU from the staged reference sources)
         on a 4e9-wide slice of the same range, process start to exit, its
         factor lines and prime count/sum compared with this library's.
other_workloads: the small Proth range in full, a 62-bit Riesel slice, a
         2e6-wide large-n range (threads per prime), a twin slice beside the
         reference's own twin GPU program, and a slice with an input sieve file.
--impl reference: the reference's own CPU path (main.c, sieve.c, pps/app.c,
         pps/factor_proth.c compiled on this host from the staged reference
         sources; every prime re-walked by pps/app.c's test_one_p) on all host
         cores (-t), one bounded sample of the same workload per step; the C
         restatement in oracle/ where the reference was not built here.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "psieve-cuda_gb300"))

METRIC = "primes/sec & n-steps/sec, k<10^4 n 2M–3M; batched vs plain GPU; serve p50/p99"
LARGE_N = dict(pmin=42 * 10**12, pmax=42 * 10**12 + 10**11, kmin=1201, kmax=9999, nmin=2000000,
          nmax=3000000)
SPAN = 1 << 31
WORKLOAD = ("large-n Proth: p in [4.2e13, 4.2e13+1e11), odd k in [1201, 9999], "
            "n in [2e6, 3e6); one step = one 2^31-wide p slice")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def shard_slices(total: int, ws: int, rank: int) -> list[int]:
    """The p slices rank `rank` of `ws` walks: r, r+ws, r+2ws, ... (independent
    units; no exchange between ranks in the data path)."""
    return list(range(rank, total, ws))


def reduce_over_ranks(x: float, op: str, ws: int, device: str) -> float:
    """max or sum of a per-rank scalar (timing and counts only) through the
    process group; the identity when ws == 1."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _traffic_from_profile(kernel: str) -> float | None:
    """DRAM bytes per prime of the walk kernel from the committed ncu summary of
    that kernel (the walk reads each prime's 16 B once, whatever the n range)."""
    f = ROOT / "profiles" / f"{kernel}_large_n.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_prime:"):
            return float(line.split(":")[1])
    return None


def _measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return json.loads(f.read_text())
    except Exception:
        return {}


def cpu_sample(seconds_target: float = 10.0, nthreads: int | None = None) -> dict:
    """Time the CPU restatement of the reference path on a bounded sample of the
    workload (a p sub-range at the start of its range)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    nthreads = nthreads or oracle.threads()
    width = 2 * 10**6
    while True:
        spec = dict(LARGE_N, pmax=LARGE_N["pmin"] + width)
        p = oracle.normalize(**spec)
        t0 = time.perf_counter()
        _, count, _ = oracle.run(p, nthreads)
        dt = time.perf_counter() - t0
        if dt >= seconds_target * 0.5 or width >= 10**9:
            break
        width = int(width * min(8.0, max(1.5, seconds_target / max(dt, 1e-3))))
    steps = (LARGE_N["nmax"] - LARGE_N["nmin"] + p.nstep - 1) // p.nstep
    return {"value": count / dt, "unit": "primes/s", "cores": nthreads, "kind": "port",
            "sample": f"p in [4.2e13, 4.2e13+{width}) = {count} primes, full n range, "
                      f"{dt:.2f} s on {nthreads} threads",
            "n_steps_per_sec": count * steps / dt, "seconds": dt, "primes": count}


REF_BIN = ROOT / "oracle" / "_ref" / "ppsieve_ref_all"
FP_RE = re.compile(r"count=(\d+),sum=0x([0-9a-f]+)")


def reference_sample(seconds_target: float = 10.0, nthreads: int | None = None,
                     width: int | None = None) -> dict | None:
    """Time the reference's OWN CPU path -- its main.c, sieve.c, pps/app.c and
    pps/factor_proth.c, built on this host from the staged reference sources
    (oracle/_ref/ppsieve_ref_all: every prime flagged, so the reference's CPU
    re-walk test_one_p runs over every prime and all n) -- on a bounded p
    sub-range at the start of the workload's range, with `nthreads` threads
    (-t).  None where the reference could not be built here."""
    import tempfile

    if not REF_BIN.exists():
        return None
    nthreads = nthreads or (len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count())
    fixed = width is not None
    width = width or 2 * 10**6
    while True:
        lo = LARGE_N["pmin"]
        with tempfile.TemporaryDirectory() as td:
            cmd = [str(REF_BIN), f"-p{lo}", f"-P{lo + width}", "-k1201", "-K9999", "-n2000000", "-N3000000",
                   f"-t{nthreads}", "-m1024", "-c1000000", "-r1000000", "-q", "-fout.txt"]
            t0 = time.perf_counter()
            r = subprocess.run(cmd, cwd=td, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
            dt = time.perf_counter() - t0
        m = FP_RE.search(r.stderr)
        if r.returncode != 0 or not m:
            return None
        count = int(m.group(1))
        if fixed or dt >= seconds_target * 0.5 or width >= 10**9:
            break
        width = int(width * min(8.0, max(1.5, seconds_target / max(dt, 1e-3))))
    steps = (LARGE_N["nmax"] - LARGE_N["nmin"] + 31) // 32
    return {"value": count / dt, "unit": "primes/s", "cores": nthreads, "kind": "reference",
            "sample": f"p in [4.2e13, 4.2e13+{width}) = {count} primes, full n range, {dt:.2f} s wall "
                      f"(process start to exit) with -t{nthreads}; the reference's main.c/sieve.c/pps/app.c "
                      f"built on this host, every prime re-walked by its CPU path",
            "n_steps_per_sec": count * steps / dt, "seconds": dt, "primes": count, "width": width}


REF_CUDA_BIN = ROOT / "oracle" / "_ref" / "ppsieve_ref_cuda"
REF_CUDA_TWIN_BIN = ROOT / "oracle" / "_ref" / "tpsieve_ref_cuda"


def _spec_args(spec: dict) -> list[str]:
    """The reference's command-line options of a job spec (main.c / pps/app.c)."""
    args = [f"-p{spec['pmin']}", f"-P{spec['pmax']}", f"-k{spec['kmin']}", f"-K{spec['kmax']}",
            f"-n{spec['nmin']}", f"-N{spec['nmax']}"]
    return args + (["-R"] if spec.get("sign") == -1 else [])


DROPIN_BIN = ROOT / "oracle" / "_ref" / "ppsieve_gpu"


def reference_gpu_sample(eng, width: int = 4 * 10**9, spec: dict | None = None, twin: bool = False,
                         binary: Path | None = None, threads: int = 1) -> dict | None:
    """The reference's OWN GPU program -- its main.c, sieve.c, pps/app.c and CUDA
    kernels pps/appcu.cu, built for this GPU from the staged reference sources
    (oracle/_ref/ppsieve_ref_cuda; tpsieve_ref_cuda, its twin build, for a twin
    job) -- on `spec` (default [4.2e13, 4.2e13 + width) of the large-n Proth
    range), process start to exit, with its factor lines and prime count/sum
    checked against this library's for the same job.  None where it was not
    built here."""
    import tempfile

    import ppsgpu

    binary = binary or (REF_CUDA_TWIN_BIN if twin else REF_CUDA_BIN)
    if not binary.exists():
        return None
    spec = spec or dict(LARGE_N, pmax=LARGE_N["pmin"] + width)
    with tempfile.TemporaryDirectory() as td:
        cmd = [str(binary), *_spec_args(spec), f"-t{threads}", "-q", "-fout.txt"]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, cwd=td, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True,
                               timeout=900)
        except (subprocess.TimeoutExpired, OSError) as ex:
            return {"unavailable": f"{binary.name}: {type(ex).__name__}"}
        dt = time.perf_counter() - t0
        out = Path(td) / "out.txt"
        lines = sorted(l.strip() for l in out.read_text().splitlines() if "|" in l) if out.exists() else []
    m = FP_RE.search(r.stderr)
    if r.returncode != 0 or not m:
        return {"unavailable": f"exit {r.returncode}: {r.stderr.strip()[-200:]}"}
    count, psum = int(m.group(1)), int(m.group(2), 16)
    fac, st = eng.run_job(ppsgpu.normalize(**dict(spec, sign=ppsgpu.PPS_SIGN_TWIN) if twin else spec))
    ours = sorted(ppsgpu.format_line(*t) for t in ppsgpu.factors_to_tuples(fac))
    what = ("the reference's main.c/sieve.c with this library's plugin (libppsgpu_app.so) in place of "
            "pps/app.c + pps/appcu.cu" if binary == DROPIN_BIN else
            "the reference's main.c/sieve.c/pps/app.c and its CUDA kernels (pps/appcu.cu) built for this GPU")
    kind = ("drop-in: the reference's main.c and sieve.c with this library's plugin" if binary == DROPIN_BIN
            else "reference GPU program" + (" (twin build)" if twin else ""))
    return {"value": count / dt, "unit": "primes/s", "kind": kind,
            "sample": f"p in [{spec['pmin']}, {spec['pmax']}) = {count} primes, n in [{spec['nmin']}, "
                      f"{spec['nmax']}), {dt:.2f} s wall (process start to exit) with -t{threads}; {what}",
            "seconds": dt, "primes": count, "factors": len(lines),
            "identical_to_ours": bool(lines == ours and st.primes == count and st.prime_sum == psum)}


def baseline_sample(seconds_target: float) -> dict:
    """The CPU baseline: the reference's own CPU path where it was built here,
    with the restatement's rate beside it; the restatement alone otherwise."""
    port = cpu_sample(seconds_target)
    ref = reference_sample(seconds_target)
    if ref is None:
        return port
    ref["port"] = {k: port[k] for k in ("value", "cores", "sample")}
    return ref


def run_mixed(eng, count: int = 512, seed: int = 1) -> dict:
    """The mixed-job workload: `count` heterogeneous jobs from `seed`, as plain one-job
    runs (pps_run_job each) and as one batched persistent run (pps_run_batch);
    the per-job results must be identical."""
    import numpy as np

    import ppsgpu

    jobs, meta = ppsgpu.mixed_jobs(seed=seed, count=count)
    repaired = sum(1 for m in meta if m[1])
    # warm-up of both forms (kernel tuning for both step classes, graph capture)
    warm = [j for j in jobs if j.step == 32][:2] + [j for j in jobs if j.step < 32][:2]
    for jp in warm:
        eng.run_job(jp)
    eng.run_batch(jobs[: min(len(jobs), 64)])
    t0 = time.perf_counter()
    plain, plain_primes, pst = [], 0, []
    for jp in jobs:
        fac, st = eng.run_job(jp)
        plain.append(fac)
        plain_primes += st.primes
        pst.append(st)
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    per, bst = eng.run_batch(jobs)
    t_batch = time.perf_counter() - t0
    # the plain form again, its tuner now warm for every kind of job in the mix
    t0 = time.perf_counter()
    plain_warm = [eng.run_job(jp)[0] for jp in jobs]
    t_plain_warm = time.perf_counter() - t0
    # where the time goes: device time per phase, the rest is host turns
    # (launches, syncs, copies, tuning) and, for the plain form, the tuner's runs
    sieve = sum(x.sieve_ms for x in pst)
    walk = sum(x.walk_ms for x in pst)
    filt = sum(x.filter_ms for x in pst)
    breakdown = {
        "plain": {"sieve_ms": sieve, "walk_ms": walk, "filter_ms": filt,
                  "other_ms": t_plain * 1e3 - sieve - walk - filt,
                  "walk_steps_per_s": sum(x.steps for x in pst) / (walk * 1e-3)},
        "batched": {"sieve_ms": bst.sieve_ms, "walk_ms": bst.walk_ms, "filter_ms": bst.filter_ms,
                    "other_ms": t_batch * 1e3 - bst.sieve_ms - bst.walk_ms - bst.filter_ms,
                    "walk_steps_per_s": bst.steps / (bst.walk_ms * 1e-3) if bst.walk_ms else None}}
    # the plain form's walk rate per kind of job (32-bit steps or shorter; n range)
    classes = {}
    for jp, x in zip(jobs, pst):
        key = f"{'s32' if jp.step == 32 else 's<32'}_{'n<1e4' if jp.nmax - jp.nmin < 10**4 else 'n>=1e4'}"
        c = classes.setdefault(key, {"jobs": 0, "steps": 0, "walk_ms": 0.0, "other_ms": 0.0})
        c["jobs"] += 1
        c["steps"] += x.steps
        c["walk_ms"] += x.walk_ms
        c["other_ms"] += x.total_ms - x.walk_ms
    for c in classes.values():
        c["walk_steps_per_s"] = c["steps"] / (c["walk_ms"] * 1e-3) if c["walk_ms"] else None
    breakdown["plain_by_kind"] = classes
    identical = (len(per) == len(plain) == len(plain_warm) and
                 all(np.array_equal(a, b) and np.array_equal(a, c) for a, b, c in zip(per, plain, plain_warm)))
    job_primes, job_sums = eng.batch_job_primes(len(jobs))
    checked = {"jobs": jobs, "lists": per, "job_primes": job_primes, "job_sums": job_sums}
    return checked, {"workload": f"{count} mixed jobs, seed {seed} (the mixed-job distribution); {repaired} "
                        "jobs had pmin raised to meet the reference's 2^(64-nstep) <= pmin rule",
            "primes": int(bst.primes), "steps": int(bst.steps), "factors": int(bst.factors),
            "plain_s": t_plain, "batched_s": t_batch,
            "plain_primes_per_s": plain_primes / t_plain, "batched_primes_per_s": bst.primes / t_batch,
            "speedup": t_plain / t_batch, "identical_results": bool(identical),
            "plain_warm_s": t_plain_warm, "speedup_vs_warm_plain": t_plain_warm / t_batch,
            "plain_note": "plain_s: one pps_run_job per job, the walk tuner timing each new kind of job "
                          "as it meets it; plain_warm_s: the same jobs again with every kind tuned",
            "waves": int(bst.waves), "chunk": int(bst.chunk), "unroll": int(bst.unroll),
            "primes_per_lane": int(bst.primes_per_lane),
            "batched_n_steps_per_s": bst.steps / t_batch, "breakdown": breakdown}


def run_other_workloads(eng) -> dict:
    """The small Proth range in full and one 2^31-wide slice of the 62-bit Riesel range through pps_run_job,
    timed after one warm-up run each (walk tuning per step class)."""
    import ppsgpu

    out = {}
    cases = {
        "small_proth_full": dict(pmin=10**12, pmax=10**12 + 2 * 10**8, kmin=1201, kmax=9999, nmin=2000,
                             nmax=3000),
        "riesel62_slice": dict(pmin=(1 << 62) - (1 << 34), pmax=(1 << 62) - (1 << 34) + SPAN, kmin=3,
                              kmax=9999, nmin=100000, nmax=1000000, sign=-1),
    }
    for name, spec in cases.items():
        jp = ppsgpu.normalize(**spec)
        eng.run_job(jp)
        t0 = time.perf_counter()
        fac, st = eng.run_job(jp)
        dt = time.perf_counter() - t0
        out[name] = {"primes": int(st.primes), "seconds": dt, "primes_per_s": st.primes / dt,
                     "n_steps_per_s": st.steps / dt, "factors": len(fac), "nstep": int(jp.nstep),
                     "walk_step": int(jp.step), "variant": int(st.variant), "split": int(st.split),
                     "phase_ms": {"sieve": st.sieve_ms, "walk": st.walk_ms, "filter": st.filter_ms,
                                  "device_total": st.total_ms}}
    # Few primes, long n: p in [4.2e13, 4.2e13 + 2e6) holds 63,903 primes, about
    # a quarter of a wave of the walk's resident threads.  The chosen threads
    # per prime against one thread per prime (forced), each timed after a
    # warm-up.
    jp = ppsgpu.normalize(**dict(LARGE_N, pmax=LARGE_N["pmin"] + 2 * 10**6))
    import numpy as np

    res, lists = {}, {}
    for label, split in (("split_1", 1), ("tuned", 0)):
        eng.set_split(split)
        eng.run_job(jp)
        t0 = time.perf_counter()
        fac, st = eng.run_job(jp)
        dt = time.perf_counter() - t0
        res[label] = {"split": int(st.split), "seconds": dt, "walk_ms": st.walk_ms,
                      "n_steps_per_s": st.steps / dt, "walk_steps_per_s": st.steps / (st.walk_ms * 1e-3),
                      "factors": len(fac)}
        lists[label] = fac
    eng.set_split(0)
    out["large_n_small_range"] = {"p_range": [jp.pmin, jp.pmax], "primes": int(st.primes), **res,
                                  "speedup": res["split_1"]["seconds"] / res["tuned"]["seconds"],
                                  "identical_results": bool(np.array_equal(lists["split_1"], lists["tuned"]))}
    out["twin_large_n_slice"] = run_twin_slice(eng)
    out["input_file_slice"] = run_input_file_slice(eng)
    return out


def run_twin_slice(eng) -> dict:
    """A twin job (both k*2^n+1 and k*2^n-1 from one walk, the reference's
    tpsieve build) on a 2^30-wide slice of the large-n range, k == 3 (mod 6) in
    [3, 9999], timed after a warm-up; beside it the reference's own twin GPU
    program on the same job, its lines checked against these."""
    import ppsgpu

    spec = dict(LARGE_N, pmax=LARGE_N["pmin"] + (1 << 30), kmin=3)
    jp = ppsgpu.normalize(**dict(spec, sign=ppsgpu.PPS_SIGN_TWIN))
    eng.run_job(jp)
    t0 = time.perf_counter()
    fac, st = eng.run_job(jp)
    dt = time.perf_counter() - t0
    return {"p_range": [jp.pmin, jp.pmax], "k": [int(jp.kmin), int(jp.kmax), int(jp.kstep)],
            "primes": int(st.primes), "seconds": dt, "primes_per_s": st.primes / dt,
            "n_steps_per_s": st.steps / dt, "walk_step": int(jp.step), "factors": len(fac),
            "reference_gpu": reference_gpu_sample(eng, spec=spec, twin=True)}


def run_input_file_slice(eng, candidates: int = 10**6) -> dict:
    """An input sieve file (-i, NewPGen format) as the output rule: `candidates`
    seeded (k, n) pairs of the large-n range's k and n ranges, on a 2^30-wide
    slice, against the same slice with the small-prime filter.  Checks: every
    line of the file run has its (k, n) in the file, and every line of the
    other run whose (k, n) is in the file is in the file run too."""
    import tempfile

    import numpy as np

    import ppsgpu

    rng = np.random.default_rng(11)
    ks = rng.integers(1201 // 2, 9999 // 2 + 1, size=candidates) * 2 + 1
    ns = rng.integers(LARGE_N["nmin"], LARGE_N["nmax"], size=candidates)
    order = np.lexsort((ks, ns))
    spec = dict(LARGE_N, pmax=LARGE_N["pmin"] + (1 << 30))
    res = {}
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "sieve.txt"
        with open(path, "w") as f:
            f.write("30:P:1:2:1\n")
            f.writelines(f"{k} {n}\n" for k, n in zip(ks[order].tolist(), ns[order].tolist()))
        # k and n bounds from the file (the reference scans a NewPGen file only
        # when one of them is left open, pps/app.c:97, 424-434)
        inp = ppsgpu.InputFile(path, pmin=spec["pmin"], pmax=spec["pmax"])
        jp = ppsgpu.normalize(**inp.spec)
        for label, use in (("small_prime_filter", None), ("input_file", inp)):
            eng.set_input(use)
            eng.run_job(jp)
            t0 = time.perf_counter()
            fac, st = eng.run_job(jp)
            dt = time.perf_counter() - t0
            res[label] = {"seconds": dt, "primes_per_s": st.primes / dt, "factors": len(fac),
                          "filter_ms": st.filter_ms, "lines": set(ppsgpu.factors_to_tuples(fac))}
        eng.set_input(None)
    in_file = set(zip(ks.tolist(), ns.tolist()))
    got, other = res["input_file"].pop("lines"), res["small_prime_filter"].pop("lines")
    ok = all((k, n) in in_file for _, k, n, _ in got) and all(t in got for t in other if (t[1], t[2]) in in_file)
    return {"p_range": [jp.pmin, jp.pmax], "candidates": candidates, **res, "consistent_with_file": bool(ok)}


def _serve_rate(srv, pool, nxt: int, rng, rate: float, window: float, max_jobs: int, served: list,
                capacity: float | None = None) -> tuple:
    """Poisson arrivals at `rate` jobs/s for `window` seconds or `max_jobs` jobs,
    whichever ends first, then every job waited for.  Latency = submission to
    result ready (the serving loop's own clock).  With `capacity` (walk steps/s
    of the whole GPU), each job's wait = latency - its own walk at that rate."""
    import numpy as np

    ids, jps = [], []
    t0 = time.perf_counter()
    t = 0.0
    while len(ids) < max_jobs:
        t += float(rng.exponential(1.0 / rate))
        if t > window:
            break
        delay = t0 + t - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        jps.append(pool[nxt % len(pool)])
        ids.append(srv.submit(jps[-1]))
        nxt += 1
    submit_s = time.perf_counter() - t0
    lat, work, primes, factors = [], [], 0, 0
    for jid, jp in zip(ids, jps):
        fac, res = srv.wait(jid)
        served.append((jp, fac))
        lat.append(res.latency_ms)
        work.append(res.primes * ((jp.nmax - jp.nmin + jp.step - 1) // jp.step))
        primes += res.primes
        factors += len(fac)
    elapsed = time.perf_counter() - t0

    def rank(v, q):
        v = sorted(v)
        return v[max(1, int(np.ceil(q * len(v)))) - 1] if v else None

    # the half of the jobs with the least walk work: what a wave cut bounds
    # (the largest jobs' latency is mostly their own walk)
    med = rank(work, 0.5) if work else 0
    small = [l for l, w in zip(lat, work) if w <= med]
    waits = [l - 1e3 * w / capacity for l, w in zip(lat, work)] if capacity else []
    extra = {"wait_p50_ms": rank(waits, 0.50), "wait_p99_ms": rank(waits, 0.99)} if capacity else {}
    return nxt, {**extra, "rate_jobs_per_s": rate, "jobs": len(ids), "offered_s": submit_s, "seconds": elapsed,
                 "achieved_jobs_per_s": len(ids) / elapsed, "primes_per_s": primes / elapsed,
                 "n_steps_per_s": sum(work) / elapsed, "factors": factors,
                 "p50_ms": rank(lat, 0.50), "p99_ms": rank(lat, 0.99), "max_ms": max(lat) if lat else None,
                 "small_half_p50_ms": rank(small, 0.50), "small_half_p99_ms": rank(small, 0.99)}


def run_serving(rates=(10.0, 30.0, 100.0, 300.0, 1000.0), window: float = 4.0, max_jobs: int = 400,
                long_rate: float = 30.0, long_window: float = 60.0, seed: int = 3,
                capacity: float | None = None) -> tuple:
    """The serving loop (pps_server_*): Poisson arrivals of jobs from the
    mixed-job distribution at each rate for `window` seconds or `max_jobs`
    jobs (so the rates above capacity, where a queue builds, still end), then
    one `long_window`-second window at `long_rate` (below capacity).  Reports
    per rate the aggregate primes/s and walk steps/s (first submission to last
    result) and the p50/p99 latency of all jobs and of the smaller half by
    walk work, and (given `capacity`, the batched form's walk steps/s) of each
    job's wait: its latency less its own walk at that rate, the delay the
    serving loop adds.  Returns ((job, factors) of every served job, summary)."""
    import numpy as np

    import ppsgpu

    need = int(sum(min(r * window * 1.3 + 16, max_jobs) for r in rates) + long_rate * long_window * 1.3) + 64
    pool, _ = ppsgpu.mixed_jobs(seed=seed, count=need)
    rng = np.random.default_rng(seed)
    per_rate, served = [], []
    with ppsgpu.Server(0) as srv:
        for jp in pool[:8]:  # warm-up: walk tuning, graph capture, sieving primes
            srv.wait(srv.submit(jp))
        nxt = 8
        for rate in rates:
            nxt, r = _serve_rate(srv, pool, nxt, rng, rate, window, max_jobs, served, capacity)
            per_rate.append(r)
        long = None
        if long_window > 0:
            nxt, long = _serve_rate(srv, pool, nxt, rng, long_rate, long_window, 1 << 30, served, capacity)
        st = srv.stats()
    return served, {"workload": f"Poisson arrivals, {window:g} s or {max_jobs} jobs per rate, then "
                                f"{long_window:g} s at {long_rate:g} jobs/s; jobs of the mixed-job distribution "
                                f"(seed {seed}); waves cut at 4e10 walk steps",
                    "rates": per_rate, "long_window": long, "waves": int(st.waves), "busy_ms": st.busy_ms,
                    "completed": int(st.completed), "failed": int(st.failed)}


RIESEL62 = dict(pmin=(1 << 62) - (1 << 34), pmax=1 << 62, kmin=3, kmax=9999, nmin=100000, nmax=1000000,
                sign=-1)


class Checker:
    """The oracle as the checker of what the GPU reported (run after the timed
    regions, never timed, never the thing measured): per-line verification of
    factor lists (p prime, p | k*2^n+c, k and n in range, the output rule) and
    the prime count/sum of whole p ranges against the oracle's sieve, on the
    host cores in a background thread, so that it overlaps the GPU's full-range
    runs."""

    def __init__(self, nthreads: int | None = None):
        from concurrent.futures import ThreadPoolExecutor

        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle

        self.ora = oracle
        self.nthreads = nthreads or max(1, oracle.threads() - 1)
        self.ex = ThreadPoolExecutor(1)
        self.verify_futs: dict[str, list] = {}
        self.fp_futs: dict[str, list] = {}

    def params(self, jp):
        """The oracle's own normalisation of a job (idempotent on normalised jobs)."""
        return self.ora.normalize(pmin=jp.pmin, pmax=jp.pmax, kmin=jp.kmin, kmax=jp.kmax, nmin=jp.nmin,
                                  nmax=jp.nmax, sign=jp.sign, kstep=jp.kstep, koffset=jp.koffset,
                                  qmax=jp.qmax)

    def verify(self, label: str, jobs_and_lists) -> None:
        """Queue the per-line verification of (job, factors) pairs under `label`."""
        import numpy as np

        jobs, rows, job_of = [], [], []
        for jp, fac in jobs_and_lists:
            jobs.append(self.params(jp))
            rows.append(fac)
            job_of.append(np.full(len(fac), len(jobs) - 1, dtype=np.uint32))
        if not jobs:
            return
        allrows = np.concatenate(rows) if rows else np.zeros(0)

        def work():
            fails, bad = self.ora.verify_factors(jobs, allrows, np.concatenate(job_of), self.nthreads)
            return {"lines": int(len(allrows)), "failures": fails,
                    "first_failures": [[int(allrows[i]["p"]), int(allrows[i]["k"]), int(allrows[i]["n"]),
                                        int(allrows[i]["c"]), int(bad[i])] for i in np.nonzero(bad)[0][:5]]}

        self.verify_futs.setdefault(label, []).append(self.ex.submit(work))

    def fingerprint(self, label: str, lo: int, hi: int, qmax: int, got_count: int, got_sum: int) -> None:
        """Queue the oracle's count/sum of [lo, hi) against the GPU's."""

        def work():
            cnt, sm = self.ora.fingerprint(lo, hi, qmax, self.nthreads)
            return {"equal": cnt == got_count and sm == (got_sum & (2**64 - 1)), "count": cnt}

        self.fp_futs.setdefault(label, []).append(self.ex.submit(work))

    def results(self) -> dict:
        out = {}
        for label in sorted(set(self.verify_futs) | set(self.fp_futs)):
            r = {}
            vs = [f.result() for f in self.verify_futs.get(label, [])]
            if vs:
                r["verified_factors"] = sum(v["lines"] for v in vs)
                r["verify_failures"] = sum(v["failures"] for v in vs)
                first = [x for v in vs for x in v["first_failures"]][:5]
                if first:
                    r["first_failures"] = first
            fs = [f.result() for f in self.fp_futs.get(label, [])]
            if fs:
                r["fingerprints_checked"] = len(fs)
                r["fingerprints_equal"] = all(f["equal"] for f in fs)
                r["oracle_primes"] = sum(f["count"] for f in fs)
            out[label] = r
        self.ex.shutdown()
        return out


def run_full_range(eng, chk: Checker, spec: dict, label: str) -> tuple[dict, dict]:
    """One workload over its whole p range, one 2^31-wide slice per pps_run_job
    call: every slice's factors go to the checker's per-line verification and
    every slice's prime count/sum to its fingerprint.  Returns the factor list of
    each slice (by index) and a summary."""
    import ppsgpu

    lists, primes, factors, gpu_s = {}, 0, 0, 0.0
    nslices = (spec["pmax"] - spec["pmin"] + SPAN - 1) // SPAN
    for i in range(nslices):
        lo = spec["pmin"] + i * SPAN
        hi = min(spec["pmax"], lo + SPAN)
        jp = ppsgpu.normalize(**dict(spec, pmin=lo, pmax=hi))
        t0 = time.perf_counter()
        fac, st = eng.run_job(jp)
        gpu_s += time.perf_counter() - t0
        lists[i] = fac
        primes += st.primes
        factors += len(fac)
        chk.verify(label, [(jp, fac)])
        chk.fingerprint(label, jp.pmin, jp.pmax, jp.qmax, st.primes, st.prime_sum)
    return lists, {"p_range": [spec["pmin"], spec["pmax"]], "slices": nslices, "primes": primes,
                   "factors": factors, "gpu_s": gpu_s}


def run_reference(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    per_step = []
    # each step one bounded sample, sized once so that the whole run stays
    # within a few minutes
    target = min(args.ref_seconds, 150.0 / (args.warmup + args.steps))
    width = None
    for i in range(args.warmup + args.steps):
        r = reference_sample(seconds_target=target, width=width)
        if r is None:
            r = cpu_sample(seconds_target=target)
        else:
            width = r["width"]
        if i >= args.warmup:
            per_step.append(r)
    value = statistics.median(r["value"] for r in per_step)
    ms = statistics.median(r["seconds"] for r in per_step) * 1e3
    last = per_step[-1]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "primes/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (deterministic p range of the configuration)",
            "config": {"workload": WORKLOAD, "sample": last["sample"]},
            "cpu_baseline": {"value": value, "unit": "primes/s", "cores": last["cores"],
                             "kind": last["kind"], "sample": last["sample"]},
            "e2e": {"value": value, "unit": "primes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "n_steps_per_sec": statistics.median(r["n_steps_per_sec"] for r in per_step)}
    print(json.dumps(line), flush=True)


def run_checks(eng, args, slice_params, seq, timed_lists, e2e_lists, mixed, served) -> dict:
    """The checker leg (after every timed leg; not timed): the large-n Proth
    workload and the 62-bit Riesel workload run in full on the GPU, every
    factor the bench reported (full runs, timed slices, the host-buffer path,
    the 512-job mix, the served jobs) is verified line by line by the oracle,
    and the prime count/sum of every full-range slice and of a seeded subset of
    the mixed jobs is compared with the oracle's sieve."""
    import numpy as np

    chk = Checker()
    out = {}
    # the lists gathered so far first, so the host cores start at once
    timed = [(slice_params(seq[args.warmup + i]), f) for i, f in enumerate(timed_lists)]
    chk.verify("large_n_timed_slices", timed)
    if e2e_lists is not None:
        chk.verify("large_n_host_buffers", [(slice_params(seq[args.warmup + i]), f)
                                            for i, f in enumerate(e2e_lists)])
    if mixed is not None:
        chk.verify("mixed_jobs", list(zip(mixed["jobs"], mixed["lists"])))
        rng = np.random.default_rng(11)
        for j in sorted(rng.choice(len(mixed["jobs"]), size=min(16, len(mixed["jobs"])), replace=False)):
            jp = mixed["jobs"][j]
            chk.fingerprint("mixed_jobs", jp.pmin, jp.pmax, jp.qmax, int(mixed["job_primes"][j]),
                            int(mixed["job_sums"][j]))
    if served is not None:
        chk.verify("served_jobs", served)
    full2, out["large_n_full"] = run_full_range(eng, chk, LARGE_N, "large_n_full")
    _, out["riesel62_full"] = run_full_range(eng, chk, RIESEL62, "riesel62_full")
    # the timed slices and the host-buffer path gave the same lists as the full run
    out["large_n_timed_slices"] = {"slices": len(timed_lists), "identical_to_full_run": all(
        np.array_equal(f, full2[seq[args.warmup + i]]) for i, f in enumerate(timed_lists))}
    if e2e_lists is not None:
        out["large_n_host_buffers"] = {"slices": len(e2e_lists), "identical_to_full_run": all(
            np.array_equal(f, full2[seq[args.warmup + i]]) for i, f in enumerate(e2e_lists))}
    t0 = time.perf_counter()
    res = chk.results()
    for label, r in res.items():
        out.setdefault(label, {}).update(r)
    out["checker"] = {"threads": chk.nthreads, "wait_after_gpu_s": time.perf_counter() - t0,
                      "what": "per line: p prime (deterministic Miller-Rabin), p | k*2^n+c, k and n in "
                              "the job's ranges with k == koffset (mod kstep), the job's side, no prime "
                              "factor below 32768; per range: prime count and sum of the oracle's sieve"}
    return out


def run_gpu(args) -> None:
    import ctypes

    import numpy as np
    import torch

    import ppsgpu

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    lib = ppsgpu.load()
    eng = ppsgpu.Engine(local)
    eng.set_batch_span(SPAN)
    if args.walk_variant >= 0:
        # a fixed walk kernel (for profiling runs, whose timing would sway the tuner)
        eng.set_variant(args.walk_variant)

    def slice_params(i: int):
        lo = LARGE_N["pmin"] + i * SPAN
        hi = min(LARGE_N["pmax"], lo + SPAN)
        return ppsgpu.normalize(**dict(LARGE_N, pmin=lo, pmax=hi))

    total_slices = (LARGE_N["pmax"] - LARGE_N["pmin"] + SPAN - 1) // SPAN
    my_slices = shard_slices(total_slices, ws, rank)
    need = args.warmup + args.steps
    seq = [my_slices[i % len(my_slices)] for i in range(need)]

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def max_over_ranks(x: float) -> float:
        return reduce_over_ranks(x, "max", ws, f"cuda:{local}")

    def sum_over_ranks(x: float) -> float:
        return reduce_over_ranks(x, "sum", ws, f"cuda:{local}")

    # ---- device-resident path (value)
    for i in range(args.warmup):
        eng.run_job(slice_params(seq[i]))
    barrier()
    launches0 = eng.launches
    stats = []
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        timed_lists = []
        for i in range(args.warmup, need):
            fac, st = eng.run_job(slice_params(seq[i]))
            stats.append(st)
            timed_lists.append(fac)
        barrier()
        elapsed = time.perf_counter() - t0
    launches = eng.launches - launches0
    primes = sum(s.primes for s in stats)
    steps_done = sum(s.steps for s in stats)
    walk_ms = sum(s.walk_ms for s in stats)
    sieve_ms = sum(s.sieve_ms for s in stats)
    elapsed = max_over_ranks(elapsed)
    value = sum_over_ranks(primes) / elapsed
    nsteps_rate = sum_over_ranks(steps_done) / elapsed

    # ---- end-to-end through the host-buffer C ABI (e2e)
    e2e = None
    if not args.no_e2e:
        host_sets = []
        for i in range(need):
            jp = slice_params(seq[i])
            est = int(1.2 * (jp.pmax - jp.pmin) / np.log(float(jp.pmin))) + 4096
            pr, n, _ = eng.sieve_range(jp.pmin, jp.pmax, jp.qmax, want_primes=True, cap=est)
            pin = torch.empty(n, dtype=torch.int64, pin_memory=True)
            pin.numpy().view(np.uint64)[:] = pr
            host_sets.append((jp, pin))
        for i in range(args.warmup):
            jp, pin = host_sets[i]
            eng.check_primes(jp, pin.numpy().view(np.uint64))
        barrier()
        h2d = d2h = 0
        e_primes = 0
        e_walk_ms = 0.0
        e_variants = set()
        e2e_lists = []
        t0 = time.perf_counter()
        for i in range(args.warmup, need):
            jp, pin = host_sets[i]
            fac, st = eng.check_primes(jp, pin.numpy().view(np.uint64))
            e2e_lists.append(fac)
            h2d += pin.numel() * 8
            d2h += 8 + fac.nbytes
            e_primes += st.primes
            e_walk_ms += st.walk_ms
            e_variants.add(int(st.variant))
        barrier()
        e_el = max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": sum_over_ranks(e_primes) / e_el, "unit": "primes/s",
               "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps),
               "path": "pps_check_primes (host primes in pinned memory, read in place by the walk over the "
                       "host link -> factors to host)",
               "ms_per_step": 1e3 * e_el / args.steps, "walk_ms_per_step": e_walk_ms / args.steps,
               "variants": sorted(e_variants)}
        del host_sets

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline of the walk kernel
    peak_mults = eng.imad_peak()
    mults = 3.0 * steps_done
    achieved = mults / (walk_ms * 1e-3)
    variant = stats[-1].variant if stats else 0
    kernel = ppsgpu.walk_kernel_name(variant)
    traffic = _traffic_from_profile(kernel)
    peaks = _measured_peaks()
    hbm = peaks.get("hbm_gbs")
    sieve_gbs = 16.0 * primes / (sieve_ms * 1e-3) / 1e9 if sieve_ms > 0 else None
    launches_walk = len(stats)  # one walk launch per job
    roofline = {"bound": "imad", "achieved": achieved / 1e9, "peak": peak_mults / 1e9,
                "unit": "Gmul/s", "frac": achieved / peak_mults,
                "traffic": (traffic * primes / launches_walk) if traffic else None,
                "traffic_unit": "bytes per launch (ncu DRAM bytes per prime x primes per launch)",
                "kernel": f"{kernel} (variant {variant}: {ppsgpu.walk_variant_name(variant)})",
                "peak_source": "measured in this run (pps_measure_imad_peak)",
                "work_per_unit": "3 multiplies per walk step (one prime advanced by 32 n)",
                "sieve": {"bound": "hbm", "achieved": sieve_gbs, "peak": hbm, "unit": "GB/s",
                          "frac": (sieve_gbs / hbm) if (sieve_gbs and hbm) else None,
                          "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                          "work_per_unit": "16 B written per prime (p + Montgomery constant)",
                          "p_range_per_s": (args.steps * SPAN / (sieve_ms * 1e-3)) if sieve_ms > 0 else None}}
    cpu = None if args.no_cpu else baseline_sample(args.ref_seconds)
    ref_gpu = None if args.no_cpu else reference_gpu_sample(eng)
    if ref_gpu is not None and DROPIN_BIN.exists():
        # the same range through the drop-in: the reference's own CPU sieve and
        # main loop feeding this library's plugin
        ref_gpu["dropin"] = reference_gpu_sample(eng, binary=DROPIN_BIN, threads=4)
    mixed_checked, batched = (None, None) if args.no_batched else run_mixed(eng, args.mixed_jobs)
    served, serving = (None, None) if args.no_serving else run_serving(
        window=args.serve_window, long_window=args.serve_long,
        capacity=batched["batched_n_steps_per_s"] if batched else None)
    others = None if args.no_batched else run_other_workloads(eng)
    verify = None if args.no_verify else run_checks(eng, args, slice_params, seq, timed_lists,
                                                    e2e_lists if e2e else None, mixed_checked, served)
    line = {"metric": METRIC, "value": value, "unit": "primes/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (deterministic p range of the configuration, primes made on device)",
            "config": {"workload": WORKLOAD, "slice_span": SPAN, "slices": seq[args.warmup:],
                       "primes_per_step": primes / args.steps,
                       "l2": "inputs larger than L2 (1.1 GB of primes per step), no flush",
                       "variant": stats[-1].variant if stats else None},
            "n_steps_per_sec": nsteps_rate,
            # primes x (nmax - nmin) per second: independent of the step size
            "n_values_per_sec": value * (LARGE_N["nmax"] - LARGE_N["nmin"]),
            "gpu_launches": launches,
            "phase_ms": {"sieve": sieve_ms, "walk": walk_ms,
                         "filter": sum(s.filter_ms for s in stats)},
            "factors": sum(s.factors for s in stats),
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "reference_gpu": ref_gpu,
            "clocks": clk.summary(),
            "batched": batched, "serving": serving, "other_workloads": others, "verify": verify}
    print(json.dumps(line), flush=True)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_profile(args) -> None:
    """One job on a reduced slice with a forced walk variant (for ncu captures):
    exactly one k_walk launch per job."""
    import ppsgpu

    eng = ppsgpu.Engine(0)
    eng.set_variant(args.variant)
    spec = dict(LARGE_N, pmax=LARGE_N["pmin"] + args.profile[0], nmax=LARGE_N["nmin"] + args.profile[1])
    for _ in range(args.profile_reps):
        fac, st = eng.run_job(ppsgpu.normalize(**spec))
        print(f"profile job: {st.primes} primes, {st.steps} steps, walk {st.walk_ms:.3f} ms, "
              f"{len(fac)} factors", flush=True)
    eng.close()


def run_profile_batched(args) -> None:
    """The mixed-job workload through pps_run_batch only (a warm-up batch
    of 64 jobs, then the 512 jobs once), for launch lists and captures of the
    batched kernels."""
    import ppsgpu

    eng = ppsgpu.Engine(0)
    if args.wave_segments:
        eng.set_wave_segments(args.wave_segments)  # smaller waves: less device memory (captures)
    if args.batch_walk:
        eng.set_batch_walk(*args.batch_walk)  # a fixed walk kernel (unroll, primes per lane)
    jobs, _ = ppsgpu.mixed_jobs(seed=1, count=args.mixed_jobs)
    eng.run_batch(jobs[:64])
    t0 = time.perf_counter()
    _, st = eng.run_batch(jobs)
    dt = time.perf_counter() - t0
    print(f"batched: {len(jobs)} jobs, {st.primes} primes, {st.steps} steps, {st.waves} waves, "
          f"{dt:.3f} s, {st.steps / dt:.4e} steps/s", flush=True)
    eng.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-window", type=float, default=4.0)
    ap.add_argument("--serve-long", type=float, default=60.0,
                    help="seconds of the long serving window at 30 jobs/s (0: none)")
    ap.add_argument("--no-verify", action="store_true",
                    help="skip the checker leg (full-range runs verified by the oracle)")
    ap.add_argument("--mixed-jobs", type=int, default=512)
    ap.add_argument("--profile", type=int, nargs=2, metavar=("SPAN", "NWIDTH"))
    ap.add_argument("--profile-reps", type=int, default=1)
    ap.add_argument("--variant", type=int, default=5)
    ap.add_argument("--walk-variant", type=int, default=-1,
                    help="fix the walk kernel of the large-n Proth jobs (default: tuned)")
    ap.add_argument("--profile-batched", action="store_true")
    ap.add_argument("--wave-segments", type=int, default=0,
                    help="--profile-batched: segments per wave (0: the maximum, 16384)")
    ap.add_argument("--batch-walk", type=int, nargs=2, metavar=("UNROLL", "PRIMES_PER_LANE"),
                    help="--profile-batched: force the batched walk kernel (8 or 16, 1 or 2)")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
    elif args.profile_batched:
        run_profile_batched(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
