import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SCENES = os.path.join(ROOT, "pathtracer_gb300", "scenes")
GOLDEN = os.path.join(ROOT, "tests", "golden")
REFERENCE = "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def built():
    """Builds (if stale) and returns the paths of the native libraries and the oracle."""
    from pathtracer_gb300 import build

    return build.build_all()


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "scenes"))
