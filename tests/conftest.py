import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import __graft_entry__ as _ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def tb():
    return _ge.load_package()


@pytest.fixture(scope="session")
def orc():
    return _ge.load_oracle()


@pytest.fixture(scope="session")
def exact():
    import oracle.mis_exact as m

    return m


@pytest.fixture(scope="session")
def native(tb):
    return sys.modules["tensorbranching_gb300._native"]


@pytest.fixture(scope="session")
def engine(tb):
    eng = tb.Engine()
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def engine_i32(tb):
    eng = tb.Engine(dtype="i32")
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def engine_i16(tb):
    """An f32 context whose GEMM tiles may run the exact packed-int16 form."""
    eng = tb.Engine(gemm_arith="i16x2")
    yield eng
    eng.close()
