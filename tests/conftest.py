import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))



def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    from gpueularsolver2d_gb300 import build
    build.build()
    from gpueularsolver2d_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle


def reference_mesh(name: str) -> str | None:
    """A mesh shipped with the reference checkout, if it is present here."""
    import build_ref  # oracle/build_ref.py: resolves the checkout or its staged copy
    for d in (build_ref.checkout_dir(), os.path.join(ROOT, "oracle", "_ref", "src")):
        p = os.path.join(d, name)
        if os.path.exists(p):
            return p
    return None
