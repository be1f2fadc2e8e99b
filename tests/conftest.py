import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(REPO, "treelet-prefetching-for-rt_gb300")
for p in (PKG_ROOT, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    from treelet_rt import build as b

    b.build_all()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import treelet_rt as rt

    return rt.Context(0)
