"""Build the native parts of the GB300 PPSieve library in-tree.

    python psieve-cuda_gb300/build.py            # libppsgpu.so (+ appcu compat lib, host plugin)

Outputs (git-ignored) go to psieve-cuda_gb300/_build/.  Every CUDA translation
unit is compiled for sm_103a only, in parallel, then linked with nvcc.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
OUT = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]

LIB_SOURCES = ["pps_kernels.cu", "pps_engine.cu", "pps_batch.cu", "pps_server.cu",
               "pps_noalloc.cu", "pps_input.cu"]
COMPAT_SOURCES = ["appcu_compat.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def build(verbose: bool = False) -> dict[str, Path]:
    OUT.mkdir(exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    srcs = [s for s in LIB_SOURCES + COMPAT_SOURCES if (CSRC / s).exists()]

    def compile_one(src: str) -> Path:
        obj = OUT / (Path(src).stem + ".o")
        if _stale(obj, [CSRC / src] + hdrs):
            cmd = [nv, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            _run(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = dict(zip(srcs, ex.map(compile_one, srcs)))

    lib = OUT / "libppsgpu.so"
    lib_objs = [objs[s] for s in LIB_SOURCES if s in objs]
    if _stale(lib, lib_objs):
        _run([nv, *ARCH, "-shared", "-o", str(lib), *map(str, lib_objs), "-lcudart", "-lpthread"])
    out = {"libppsgpu": lib}

    compat_objs = [objs[s] for s in COMPAT_SOURCES if s in objs]
    if compat_objs:
        clib = OUT / "libppsgpu_appcu.so"
        if _stale(clib, compat_objs + [lib]):
            _run([nv, *ARCH, "-shared", "-o", str(clib), *map(str, compat_objs),
                  f"-L{OUT}", "-lppsgpu", "-Xlinker", "-rpath,$ORIGIN", "-lcudart"])
        out["libppsgpu_appcu"] = clib

    # host plugin (the app.h hooks, include/pps_app.h) as a shared library; it
    # resolves main.c's globals (pmin, pmax, bexit, ...) from the executable
    plugin_src = HOST / "app_gpu.c"
    if plugin_src.exists():
        plib = OUT / "libppsgpu_app.so"
        deps = [plugin_src, lib] + sorted(HOST.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
        # the plugin, and its twin build (the reference's tpsieve: -DSEARCH_TWIN)
        for name, defs in (("libppsgpu_app", []), ("libppsgpu_app_twin", ["-DPPS_TWIN"])):
            plib = OUT / f"{name}.so"
            if _stale(plib, deps):
                _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-Wextra", "-fPIC", "-shared", *defs,
                      f"-I{INCLUDE}", f"-I{HOST}", str(plugin_src), "-o", str(plib), f"-L{OUT}",
                      "-lppsgpu", "-Wl,-rpath,$ORIGIN", "-lpthread"])
            out[name] = plib
    return out


if __name__ == "__main__":
    res = build(verbose="-v" in sys.argv)
    for k, v in res.items():
        print(f"{k}: {v}")
