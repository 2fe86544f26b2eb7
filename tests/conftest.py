import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import build as oracle_build

    from md_sim_gb300 import abi

    oracle_build.build()
    return abi.Lib(oracle_build.path(), "ref_")


@pytest.fixture(scope="session")
def gpulib():
    from md_sim_gb300 import build as lib_build

    import md_sim_gb300

    lib_build.build()
    return md_sim_gb300.load()
