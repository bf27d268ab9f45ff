import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    if not O.available():
        from oracle import build_ref
        build_ref.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    from slr_gb300 import api
    if not api.LIB_PATH.is_file():
        from slr_gb300 import build
        build.build()
    return api
