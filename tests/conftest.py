import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libtw_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def reflib():
    from oracle.oracle import RefLib

    if not RefLib.available():
        pytest.skip("reference sources not available to build oracle/_ref")
    try:
        return RefLib()
    except FileNotFoundError as e:
        pytest.skip(str(e))


@pytest.fixture(scope="session")
def ctx():
    """A device context; builds libtw_gb300.so first if it is missing."""
    import tetwild_gb300 as tw
    from tetwild_gb300 import build as twbuild

    if not tw.library_path().exists():
        twbuild.build()
    c = tw.Context(0)
    yield c
    c.close()


def golden(name):
    return np.load(GOLDEN / name)
