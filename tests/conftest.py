import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


@pytest.fixture(scope="session")
def r2p():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def O():
    from oracle import build_oracle, oracle
    build_oracle.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def W(r2p):
    from raw2png_gb300 import workloads
    return workloads


@pytest.fixture(scope="session")
def engine(r2p):
    eng = r2p.Engine(0)
    yield eng
    eng.close()
