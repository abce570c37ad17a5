import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "sand-water-coupling_gb300"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def swc_mod():
    import swc

    swc.load()
    return swc
