"""bench.py's host-side helpers (CPU only): the reference's command line of a
job spec, and the reference legs' absence where the reference was not built."""
from __future__ import annotations

import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_spec_args_are_the_reference_options():
    b = _bench()
    args = b._spec_args(dict(pmin=42 * 10**12, pmax=42 * 10**12 + 10**6, kmin=1201, kmax=9999, nmin=2000000,
                             nmax=3000000))
    assert args == ["-p42000000000000", "-P42000001000000", "-k1201", "-K9999", "-n2000000", "-N3000000"]
    riesel = b._spec_args(dict(pmin=10**12, pmax=10**12 + 10, kmin=3, kmax=5, nmin=100, nmax=200, sign=-1))
    assert riesel[-1] == "-R"


def test_reference_legs_absent_without_a_build(tmp_path):
    b = _bench()
    b.REF_CUDA_BIN = tmp_path / "missing"
    b.REF_CUDA_TWIN_BIN = tmp_path / "missing_twin"
    assert b.reference_gpu_sample(None) is None
    assert b.reference_gpu_sample(None, twin=True) is None
    assert b.reference_gpu_sample(None, binary=tmp_path / "missing_dropin") is None
    b.REF_BIN = tmp_path / "missing_cpu"
    assert b.reference_sample(1.0) is None
