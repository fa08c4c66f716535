import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_lib():
    """Builds (if stale) and loads libakua_pbf.so; GPU tests must run the native library."""
    from akuaengine_gb300 import build as _build
    import akuaengine_gb300 as ak

    _build.build_library()
    return ak.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.load()
    return oracle
