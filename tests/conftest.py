"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
a CPU-only host."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "d-pdlp_gb300")
for p in (PKG, os.path.join(ROOT, "tests"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)
os.environ.setdefault("PDLP_QUIET", "1")  # no per-solve summary in test logs


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def lib():
    import cupdlpx
    if not os.path.exists(cupdlpx.LIB_PATH):
        import build  # compiles the library (nvcc cross-compiles without a GPU)
        build.build()
    return cupdlpx.lib()


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib.load()


@pytest.fixture(scope="session")
def ref():
    import oracle_lib
    r = oracle_lib.load_ref()
    if r is None:
        pytest.skip("reference host code not built (needs the reference sources)")
    return r
