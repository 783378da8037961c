import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "parallel-pandapower-solver_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def grid118():
    from p3s_gb300.synthetic import grid_118

    return grid_118()


@pytest.fixture(scope="session")
def grid2000():
    from p3s_gb300.synthetic import grid_2000

    return grid_2000()
