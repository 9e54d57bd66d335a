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


def _match_lines(got, exp):
    """Match the library's line table to the oracle's rows.  The library orders lines for
    locality (direction groups, lattice tiles), the oracle by (direction, lattice point), so
    the two tables must hold the same rows as multisets; each oracle row is then located in
    the library's table by its (entry, exit, direction) key.  Returns, per oracle row, the
    library rows with that key: one row, or several where lattice points of one direction
    have lines that share entry and exit voxels (line spacing below a cell)."""
    import numpy as np

    assert got.shape == exp.shape
    order = lambda t: t[np.lexsort(t.T[::-1])]
    np.testing.assert_array_equal(order(got), order(exp))
    where = {}
    for i, r in enumerate(got[:, :3].tolist()):
        where.setdefault(tuple(r), []).append(i)
    return [where[tuple(r)] for r in exp[:, :3].tolist()]


@pytest.fixture(scope="session")
def match_lines():
    return _match_lines
