import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (HERE, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import nl2d_testlib as T
    return T.load_oracle()


@pytest.fixture(scope="session")
def gpulib():
    import psyclonebench_gb300 as P
    import torch  # noqa: F401  (only to probe for a device)
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return P.load_library()


@pytest.fixture(autouse=True)
def _fresh_library(request):
    """Every test that uses the library starts with no problem registered
    and no sticky error status left by an earlier test.
    The library keys a problem's residency on the caller's host pointers
    (the reference's driver keeps its arrays for the program's life), so a
    model whose arrays land at the addresses of an earlier test's freed
    arrays would otherwise be taken for that earlier registration."""
    if "gpulib" in request.fixturenames:
        import ctypes
        lib = request.getfixturevalue("gpulib")
        lib.nl2d_finalize()
        lib.nl2d_last_error(ctypes.create_string_buffer(256), 256)  # no status carried over
    yield
