import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    """GPU tests get a 10-minute limit where pytest-timeout is installed (the thread method
    ends the process, so a test stuck in a host wait cannot hold the GPU for longer)."""
    if not config.pluginmanager.hasplugin("timeout"):
        return
    for item in items:
        if item.get_closest_marker("gpu") and not item.get_closest_marker("timeout"):
            item.add_marker(pytest.mark.timeout(600, method="thread"))


@pytest.fixture(scope="session")
def built():
    """Builds libmhsw.so / libmhsw_gen.so / liboracle.so once per session."""
    from mhm2_staging_gb300 import build as b
    from oracle import oracle

    b.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    """A GPUDriver on device 0 with the measured scoring (1, -3, -5, -2, ambiguity -2)."""
    from mhm2_staging_gb300 import GPUDriver, get_num_node_gpus

    if get_num_node_gpus() < 1:
        pytest.fail("no CUDA device: GPU tests need a GB300")
    d = GPUDriver()
    d.init(0, 1, 1, -3, -5, -2, 300)
    d.set_ambiguity(-2)
    return d
