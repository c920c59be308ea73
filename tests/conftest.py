import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    import oracle_py
    oracle_py.build(ref=False)
    return oracle_py


@pytest.fixture(scope="session")
def fk():
    import spac_gb300
    from spac_gb300 import fk as fkmod
    if not os.path.exists(spac_gb300.LIB_PATH):
        spac_gb300.build()
    fkmod.load()
    return fkmod


@pytest.fixture(scope="session")
def host_ctx(fk):
    c = fk.Context(device=-1, seed=1)
    yield c
    c.close()


@pytest.fixture(scope="session")
def gpu(fk):
    c = fk.Context(device=0, seed=20251203)
    yield c
    c.close()
