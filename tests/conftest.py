import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def built():
    """Product library and CPU oracle, built in-tree."""
    import __graft_entry__ as ge
    from vedas_gb300 import build as vb

    vb.build()
    import subprocess

    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"], check=True)
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import vedas_gb300 as vg

    c = vg.Context(0, arena_bytes=24 << 30)
    yield c
    c.close()
