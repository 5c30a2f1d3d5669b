import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Builds the native libraries and the oracle once per session."""
    from changa_gb300 import build
    build.build_all()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def cuda_ok(built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.init()
    return True


@pytest.fixture(autouse=True)
def _record_library_errors(request):
    """GPU tests run the library with errors recorded rather than aborting
    the process, so a failing call surfaces as a test failure with its
    message."""
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    from changa_gb300 import _native as N
    N.cuda_lib().changa_gb300_set_error_mode(N.CHANGA_ERRORS_RECORD)
    yield
