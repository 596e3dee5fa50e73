import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.build(pyoracle.ref_dir())
    return pyoracle


@pytest.fixture(scope="session")
def hype():
    """The GPU package; fails (does not skip) when the library cannot be built or loaded."""
    import acoustic_petsc_gb300 as H

    H.build()
    H.lib()
    return H
