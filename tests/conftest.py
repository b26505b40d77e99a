import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libm3sph kernels)")


@pytest.fixture(scope="session")
def built_lib():
    from m3tet_sph_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def tiny():
    from m3tet_sph_gb300 import workloads as W
    return W.make_workload('tiny')


@pytest.fixture(scope="session")
def tiny_plates():
    from m3tet_sph_gb300 import workloads as W
    return W.make_workload('tiny_plates')
