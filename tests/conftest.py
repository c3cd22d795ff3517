import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    from diskdyn_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def engine(built_lib):
    from diskdyn_gb300.engine import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="session")
def refk():
    """The reference's own kernels (compiled unmodified for sm_103a) behind a runner."""
    import oracle.refk as r
    if not r.available():
        pytest.fail("reference cubin oracle/_ref/ddyn_ref_sm103a.cubin is missing")
    r.lib()
    return r
