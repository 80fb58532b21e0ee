import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def tmc_mod():
    from tiny_mc_gb300 import _build
    _build.build_library()
    import tiny_mc_gb300
    tiny_mc_gb300.lib()
    return tiny_mc_gb300


def ref_tree_available() -> bool:
    from oracle import oracle
    return os.path.isfile(os.path.join(oracle.REFERENCE_TREE, "photon.c"))
