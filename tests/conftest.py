"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on a CPU-only host.

The CPU oracle (oracle/port, and oracle/_ref where the reference tree and an x86 host
are available) is the checker; only tests import it."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def port():
    from oracle import Oracle

    return Oracle("port")


@pytest.fixture(scope="session")
def ref():
    from oracle import Oracle, ref_available

    if not ref_available():
        pytest.skip("the reference oracle builds only on x86 hosts with the reference tree")
    return Oracle("ref")


@pytest.fixture(scope="session")
def ctx():
    """A GPU context; a GPU test that cannot get one fails (it does not skip)."""
    from axiomr_gb300.api import Context

    c = Context(0)
    yield c
    c.close()
