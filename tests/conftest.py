import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built librchem_gpu.so")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def _oracle():
    """The oracle module.  RCHEM_SANITIZE_PORT names an instrumented (ASan and
    UBSan) build of oracle/pq2_port.c to load in place of the plain one;
    tests/test_sanitizers.py runs the oracle tests that way."""
    import oracle

    san = os.environ.get("RCHEM_SANITIZE_PORT")
    if san:
        oracle.PORT_SO = san
    return oracle


@pytest.fixture(scope="session")
def port():
    oracle = _oracle()
    p = oracle.port()
    p.set_boys(True)
    return p


@pytest.fixture(scope="session")
def oracle_mod():
    oracle = _oracle()
    oracle.port().set_boys(True)
    return oracle


@pytest.fixture(scope="session")
def golden_eri():
    with open(os.path.join(GOLDEN, "eri_prims.json")) as f:
        return json.load(f)["items"]


@pytest.fixture(scope="session")
def golden_onee():
    with open(os.path.join(GOLDEN, "onee_prims.json")) as f:
        return json.load(f)["items"]


def load_npz(tag):
    return dict(np.load(os.path.join(GOLDEN, tag + ".npz")))


@pytest.fixture(scope="session")
def gpu():
    """The built library on a CUDA device; builds it when missing."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from rchem_gb300 import _lib, build

    build.build()
    return _lib.lib()
