import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import subprocess
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    import kernel_cases as kc
    return kc.load_backend("oracle")


@pytest.fixture(scope="session")
def gpu_lib():
    from lakcluster_c_gb300 import build
    build.build_lib()
    import kernel_cases as kc
    return kc.load_backend("gpu")
