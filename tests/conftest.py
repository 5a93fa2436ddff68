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


def pytest_collection_modifyitems(config, items):
    """Every GPU test ends within 5 minutes: where pytest-timeout is installed, a test
    still running then has its stacks dumped and the process exits (the thread method,
    which also ends a host thread waiting on the device)."""
    if not config.pluginmanager.hasplugin("timeout"):
        return
    for item in items:
        if item.get_closest_marker("gpu") and not item.get_closest_marker("timeout"):
            item.add_marker(pytest.mark.timeout(300, method="thread"))


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
