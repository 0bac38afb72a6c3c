import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the reference's src/ tree: $IDEFIX_SRC, else a `reference/` checkout beside
# this repository (absent on machines without the reference: those tests skip)
REFERENCE_SRC = os.environ.get("IDEFIX_SRC") or os.path.join(os.path.dirname(ROOT), "reference", "src")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def oracle_lib():
    """Build (if needed) and return the path of the plain-C oracle."""
    path = os.path.join(ROOT, "oracle", "libofx.so")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "libofx.so"], check=True)
    return path


@pytest.fixture(scope="session")
def reference_libs():
    """Build the reference hot-path harness when the reference tree exists."""
    if not os.path.isdir(REFERENCE_SRC):
        pytest.skip("reference source tree not present on this machine")
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"IDEFIX_SRC={REFERENCE_SRC}"], check=True)
    return os.path.join(ROOT, "oracle", "_ref")
