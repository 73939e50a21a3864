import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_path():
    import hxtest
    return hxtest.build_oracle()


@pytest.fixture(scope="session")
def gpu_path():
    """The CUDA library; a GPU test fails loudly (it does not fall back) when the
    device or the library is missing."""
    import hxtest
    path = hxtest.build_gpu_lib()
    L = hxtest.lib(path)
    L.lib.hx_set_abort_on_error(0)
    L.lib.initialize_hommexx_session()
    code, msg = L.last_error()
    assert code == 0, f"CUDA device unavailable for the GPU tests: {msg}"
    return path


@pytest.fixture(scope="session")
def gpu_lib_cpu():
    """The CUDA library, built here and loaded without using a GPU (host-only calls)."""
    import hxtest
    return hxtest.build_gpu_lib()
