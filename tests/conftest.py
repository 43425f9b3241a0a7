import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built engine library")


@pytest.fixture(scope="session")
def torus64():
    from raptor_gb300 import synth
    return synth.make_torus(n1=64, n2=64)


@pytest.fixture(scope="session")
def torus256():
    from raptor_gb300 import synth
    return synth.make_torus(n1=256, n2=256)
