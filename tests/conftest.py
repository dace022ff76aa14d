import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SCENES = os.path.join(ROOT, "pathtracer_gb300", "scenes")
GOLDEN = os.path.join(ROOT, "tests", "golden")
# The reference tree, where it is mounted (the recipe oracle/ref_shader.py
# names its default location; PT_REFERENCE_ROOT overrides it).  Tests that
# read it skip where it is absent.
from oracle.ref_shader import reference_root  # noqa: E402

REFERENCE = reference_root()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def built():
    """Builds (if stale) and returns the paths of the native libraries and the oracle."""
    from pathtracer_gb300 import build

    return build.build_all()


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "scenes"))
