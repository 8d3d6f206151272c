import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    """The C oracle (test infrastructure), built on first use."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def engine_mod():
    """mt_gb300.engine with libmtg.so built."""
    from mt_gb300 import build, engine
    build.build()
    engine.load()
    return engine
