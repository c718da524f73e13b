import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built engine library")


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if stale) and load the CUDA engine.  No fallback: a GPU test
    fails when the library cannot be built or loaded."""
    from mphimplicit_gb300 import build, engine
    build.build()
    return engine.load_library()


@pytest.fixture(scope="session")
def oracle_built():
    import oracle as orc
    orc.build_oracle()
    return orc
