import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

# Location of the reference sources for the optional known-answer tests;
# absent on machines that only carry this repository.
REFERENCE_DIR = os.environ.get("LBX_REFERENCE_DIR", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def reference_file(rel):
    p = os.path.join(REFERENCE_DIR, rel)
    if not os.path.exists(p):
        pytest.skip("reference sources not present: %s" % rel)
    return p


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built for sm_103a; GPU tests fail loudly without it."""
    from lambrex_gb300 import build as B
    B.build()
    from lambrex_gb300 import lbx
    lbx.lambrexInit()
    return lbx
