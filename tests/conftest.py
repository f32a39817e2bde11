import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ref_lib(oracle_mod):
    lib = oracle_mod.ref_lib()
    if lib is None:
        pytest.skip("reference build (oracle/_ref) not available here")
    return lib


@pytest.fixture(scope="session")
def lgx():
    import libint_gb300
    return libint_gb300


@pytest.fixture(scope="session")
def gpu_ctx(lgx):
    ctx = lgx.Context(0)
    yield ctx
    ctx.close()
