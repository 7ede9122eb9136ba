import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "trans-omics-acceleration-library_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the libraries once if they are missing (build() is idempotent)."""
    import __graft_entry__ as g
    need = [os.path.join(PKG, "lib", "libtal_bsw.so"), os.path.join(PKG, "lib", "libtal_bsw_synth.so"),
            os.path.join(ROOT, "oracle", "_build", "liboracle_bsw.so")]
    if not all(os.path.exists(p) for p in need):
        g.build()
    yield
