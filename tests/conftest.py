import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libohpic.so")


@pytest.fixture(scope="session")
def ohpic():
    """The GPU library; built in-tree if the .so is missing (no fallback path)."""
    import ohhelppic3d_gb300 as P
    if not os.path.exists(P.LIB_PATH):
        P.build()
    P.lib()
    return P


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build()
    return O
