import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and librad_gpu.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    oracle_lib.lib()
    return oracle_lib


@pytest.fixture(scope="session")
def rad():
    """The product library on the device; fails loudly when it is missing."""
    import radiantiumplusplus_gb300 as rad
    rad.lib()
    rad.init()
    return rad


@pytest.fixture(scope="session")
def scene_dir(tmp_path_factory):
    return tmp_path_factory.mktemp("scenes")
