import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle as po

    po.build(ref=True)  # oracle/Makefile skips the reference build where its tree is absent
    return po


@pytest.fixture(scope="session")
def kmx():
    """The CUDA package, built in-tree if needed."""
    from kronmult_gb300 import build as kb

    kb.build()
    import kronmult_gb300

    kronmult_gb300.lib()
    return kronmult_gb300
