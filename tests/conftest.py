import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "staq-dic_gb300"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libstaqdic.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as orc
    return orc


@pytest.fixture(scope="session")
def ctx():
    import staqdic
    c = staqdic.Context(0)
    yield c
    c.close()
