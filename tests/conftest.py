import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")
    # build the library and the oracle once per session if they are missing
    import __graft_entry__
    if not os.path.exists(os.path.join(ROOT, "connectivity_gb300", "libgbconn.so")) or \
            not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
        __graft_entry__.build()


@pytest.fixture(scope="session")
def ctx():
    import connectivity_gb300 as gb
    c = gb.Context(0)
    yield c
    c.close()
