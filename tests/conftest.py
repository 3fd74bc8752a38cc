import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "opengjk-gpu_gb300"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built engine library")


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o
    o.build()
    return o


@pytest.fixture(scope="session")
def twin():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "tests", "twin")], check=True)
    import twin_bind
    return twin_bind


@pytest.fixture(scope="session")
def engine():
    """The GPU engine (built and loaded); GPU tests fail loudly without it."""
    from ogx import build, engine as eng
    build.build()
    return eng
