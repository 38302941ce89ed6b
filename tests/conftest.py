"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import Port

    return Port()


@pytest.fixture(scope="session")
def port_mt():
    """The oracle restatement with its per-particle loops on every host core
    (results do not depend on the thread count), for large parity cases."""
    from oracle.oracle import Port

    p = Port()
    p.set_threads(os.cpu_count() or 1)
    return p


@pytest.fixture(scope="session")
def ref():
    from oracle import build_oracle
    from oracle.oracle import Ref

    if build_oracle.build_ref() is None:
        pytest.skip("reference sources not present on this host")
    return Ref()


@pytest.fixture(scope="session")
def capi():
    from novaphy_gb300 import capi as c

    c.load()
    return c
