import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lightmetrica-v3_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs through the C-ABI")


@pytest.fixture(scope="session")
def native_lib():
    """liblmgpu.so, built in-tree if missing."""
    from lightmetrica import _native as N
    if not os.path.exists(N.LIB_PATH):
        import build_native
        build_native.build()
    return N.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def ref_mod():
    """oracle/_ref/liblmref.so: the reference's own accel and math code, compiled from its sources.
    Only where those sources are present; elsewhere the tests that need it skip."""
    from oracle import ref as R
    if not R.available():
        pytest.skip("the reference's sources are absent, so oracle/_ref is not built")
    return R


@pytest.fixture
def lm(native_lib):
    import lightmetrica as lm_
    lm_.init()
    yield lm_
    lm_.reset()
