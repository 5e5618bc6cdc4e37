import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)



def _reference_dir():
    """Location of the LAMBReX sources for the optional known-answer tests:
    LBX_REFERENCE_DIR, else a checkout named ``reference`` beside this
    repository; None when neither exists (the tests that need it skip)."""
    env = os.environ.get("LBX_REFERENCE_DIR")
    if env:
        return env
    sib = os.path.join(os.path.dirname(ROOT), "reference")
    return sib if os.path.isdir(os.path.join(sib, "tests")) else None


REFERENCE_DIR = _reference_dir()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def reference_file(rel):
    if REFERENCE_DIR is None:
        pytest.skip("reference sources not present (set LBX_REFERENCE_DIR)")
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
