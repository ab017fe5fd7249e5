import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")


@pytest.fixture(scope="session")
def oracle_lib():
    """Build the CPU oracle if it is missing (it is test infrastructure)."""
    from oracle import orc

    if not os.path.exists(orc.LIB_PATH):
        from amressif_gb300 import build as b

        b.build_oracle()
    return orc.lib()


@pytest.fixture(scope="session")
def gpu_lib():
    import amressif_gb300 as ns

    return ns.lib()
