import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "squares-in-disk_gb300")
for p in (os.path.join(PKG, "python"), PKG, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py
    oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def engine_lib():
    import sid_gb300
    if not os.path.exists(sid_gb300.LIB_PATH):
        import build as engine_build
        engine_build.build(extra_ir_dirs=[os.path.join(REPO, "tests", "golden", "kat")])
    return sid_gb300.load()


@pytest.fixture(scope="session")
def engine(engine_lib):
    import sid_gb300
    eng = sid_gb300.Engine(0)
    yield eng
    eng.close()
