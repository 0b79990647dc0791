import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on a GB300)")


@pytest.fixture(scope="session")
def built_library():
    """The GPU library and scene library, built in-tree (nvcc cross-compiles
    without a GPU)."""
    import srp_gb300
    srp_gb300.build()
    return srp_gb300.library_path()


@pytest.fixture(scope="session")
def oracle_exe():
    """The CPU oracle scene runner (test infrastructure only)."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"])
    return os.path.join(ROOT, "oracle", "_build", "port_scenes")
