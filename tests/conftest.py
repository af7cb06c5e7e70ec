import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "psieve-cuda_gb300"
ORACLE = ROOT / "oracle"
GOLDEN = ROOT / "tests" / "golden"
for p in (str(PKG), str(ORACLE), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def ora(built):
    import oracle

    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def pps(built):
    import ppsgpu

    ppsgpu.load()
    return ppsgpu


@pytest.fixture(scope="session")
def engine(pps):
    eng = pps.Engine(0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def ref_cases():
    f = GOLDEN / "ref_cases.json"
    if not f.exists():
        pytest.skip("golden fixtures not generated")
    return json.loads(f.read_text())


@pytest.fixture(scope="session")
def kat49():
    f = GOLDEN / "kat49.json"
    if not f.exists():
        pytest.skip("kat49 fixtures not generated")
    return json.loads(f.read_text())
