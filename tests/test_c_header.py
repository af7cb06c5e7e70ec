"""The public header from plain C: a C99 program that includes
include/ppsgpu.h, links libppsgpu.so and calls the entry points that need no
GPU (version, parameter normalisation with the reference's rules, checkpoint
text round trip, the allocation-failure hook, engine creation that reports a
missing GPU as a status code).  Checks that the header is valid C, not only
C++, and that a C caller sees the documented behaviour."""
from __future__ import annotations

import shutil
import subprocess

import pytest

C_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "ppsgpu.h"

int main(void) {
  printf("version %s\n", pps_version());

  /* the reference's example job: -p42070e9 -P42070050e6 -k1201 -K9999 -N2000000 */
  pps_job_spec spec;
  memset(&spec, 0, sizeof spec);
  spec.pmin = 42070000000000ull;
  spec.pmax = 42070050000000ull;
  spec.kmin = 1201;
  spec.kmax = 9999;
  spec.nmax = 2000000;
  pps_job_params jp;
  int rc = pps_normalize(&spec, &jp);
  printf("normalize %d nmin %u nmax %u kmin %llu kmax %llu step %u\n", rc, jp.nmin, jp.nmax,
         (unsigned long long)jp.kmin, (unsigned long long)jp.kmax, jp.step);

  /* a rejected job: pmin must be above 2^32 (pps/appcu.cu:236) */
  spec.pmin = 1000;
  spec.pmax = 100000;
  rc = pps_normalize(&spec, &jp);
  printf("reject %d %s\n", rc, rc == PPS_ERR_INVALID_PARAM ? "invalid" : "other");

  /* checkpoint text round trip */
  spec.pmin = 42070000000000ull;
  spec.pmax = 42070050000000ull;
  pps_normalize(&spec, &jp);
  pps_checkpoint c;
  memset(&c, 0, sizeof c);
  c.pmin = jp.pmin;
  c.p = jp.pmin + 1000000;
  c.count = 12345;
  c.sum = 0x0123456789abcdefull;
  c.nmin = jp.nmin;
  c.nmax = jp.nmax;
  c.factor_count = 3;
  char text[256];
  const int len = pps_checkpoint_format(&c, text, sizeof text);
  pps_checkpoint back;
  rc = pps_checkpoint_parse(text, &jp, &back);
  printf("checkpoint %d %d same %d\n", len > 0, rc,
         back.p == c.p && back.count == c.count && back.sum == c.sum && back.factor_count == 3);

  /* the allocation-failure hook only counts on the host */
  pps_debug_fail_allocs(0, 0);
  printf("hook %d\n", pps_debug_fail_allocs(0, 0));

  /* engine creation: a status code either way, never an exit */
  pps_engine *e = NULL;
  rc = pps_engine_create(0, &e);
  printf("engine %s\n", rc == PPS_OK ? "ok" : (rc == PPS_ERR_NO_DEVICE ? "no-device" : "error"));
  if (rc == PPS_OK) pps_engine_destroy(e);
  return 0;
}
"""


def test_header_from_c(built, pps, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "use_ppsgpu.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "use_ppsgpu"
    lib_dir = pps.LIB_PATH.parent
    root = lib_dir.parent.parent
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(root / "include"), str(src), "-o", str(exe),
                    "-L", str(lib_dir), "-lppsgpu", f"-Wl,-rpath,{lib_dir}"], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    lines = dict(line.split(" ", 1) for line in out.strip().splitlines())
    assert lines["version"].startswith("ppsgpu")
    # nmax as given; kmin and kmax already odd, so kept by the rounding of pps/app.c:705-708
    norm = lines["normalize"].split()
    assert norm[0] == "0"
    assert int(norm[4]) == 2000000 and int(norm[6]) == 1201 and int(norm[8]) == 9999
    assert lines["reject"].endswith("invalid")
    assert lines["checkpoint"] == "1 0 same 1"
    assert lines["hook"] == "0"
    assert lines["engine"] in ("ok", "no-device")
