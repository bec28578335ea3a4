import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA kernels through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (no-op when up to date)."""
    import oracle
    from umcx_gb300.build import build

    build()
    oracle.build(reference_root=None)
    yield


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLDEN / "reference_runs.json").read_text())


@pytest.fixture(scope="session")
def ctx():
    from umcx_gb300 import Context

    c = Context(0)
    yield c
    c.close()
