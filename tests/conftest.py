import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: long CPU test")


# A checkout of lyon's sources, for the tests that parse its third-party fixtures in place
# (they are never copied into this repository). Unset: those tests are skipped.
REFERENCE = os.environ.get("LYON_REFERENCE_DIR")


@pytest.fixture(scope="session")
def reference_dir():
    if not REFERENCE or not os.path.isdir(REFERENCE):
        pytest.skip("set LYON_REFERENCE_DIR to a checkout of lyon's sources")
    return REFERENCE
