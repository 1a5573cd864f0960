import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "logo-tsp-solver_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def lg():
    """The CUDA library binding; fails loudly when the library is missing."""
    import logo_gpu
    if not os.path.exists(logo_gpu.LIB_PATH):
        logo_gpu.build()
    logo_gpu.load()
    return logo_gpu


@pytest.fixture(scope="session")
def inst():
    import instances
    return instances
