import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU case")


def pytest_collection_modifyitems(config, items):
    # Run the file that exercises the allocation-free entry point last.
    items.sort(key=lambda it: 1 if os.path.basename(str(it.fspath)).startswith("test_zz") else 0)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if missing; skips when no GPU is visible."""
    import fluids_gb300
    fluids_gb300.build()
    if not fluids_gb300.cuda_available():
        pytest.skip("no CUDA device")
    return fluids_gb300
