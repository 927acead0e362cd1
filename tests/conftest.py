import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the in-tree libraries the tests use (quick, incremental)."""
    from oracle import build as obuild
    from swmapper_gb300 import _build
    _build.build_synth()
    obuild.build_oracle()
    obuild.build_ref()
    yield


@pytest.fixture(scope="session")
def cuda_lib():
    from swmapper_gb300 import _build
    _build.build_cuda()
    import swmapper_gb300 as swm
    return swm
