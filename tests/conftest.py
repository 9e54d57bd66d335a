import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "parallel-3d-pressure-reconstruction_gb300")
for p in (REPO, PKG, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    return oracle.Oracle()


@pytest.fixture(scope="session")
def reflib():
    import oracle

    path = oracle.build_ref()
    if path is None:
        pytest.skip("reference sources are not staged on this machine")
    return oracle.RefLib(path)


@pytest.fixture(scope="session")
def omni():
    import omni3d

    omni3d.build()
    omni3d.lib()
    return omni3d
