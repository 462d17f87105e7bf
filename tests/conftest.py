import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# The reference tree (niepp/astc_encoder) is read only where the environment
# names it in ASTC_REFERENCE_DIR; tests that read it skip elsewhere and the
# committed fixtures under tests/golden/ stand in.
REFERENCE = os.environ.get("ASTC_REFERENCE_DIR", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def native():
    """The product library, built in-tree if stale (no GPU needed to load it)."""
    from astc_encoder_gb300 import build
    build.build()
    import astc_encoder_gb300 as a
    a.load_library()
    return a


@pytest.fixture(scope="session")
def reference_dir():
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "textures")):
        pytest.skip("reference tree not given (set ASTC_REFERENCE_DIR)")
    return REFERENCE
