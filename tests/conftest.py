import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "masterthesis-heterogeneous-pc_gb300")
for d in (PKG, ROOT):
    if d not in sys.path:
        sys.path.insert(0, d)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu on a GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (no-op when up to date)."""
    import hpc_build

    hpc_build.build_library()
    hpc_build.build_oracle()
    yield


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)
