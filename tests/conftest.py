"""pytest configuration: the ``gpu`` marker and shared fixtures.

``-m "not gpu"`` runs the oracle against the reference's golden vectors,
the host-side library (BVH build, motion, ABI surface) and the multi-process
host logic; ``-m gpu`` runs the CUDA path against the oracle and the golden
vectors through the C ABI.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the CUDA path)")


@pytest.fixture(scope="session")
def port():
    from oracle.oracle import Port, build

    build(ref=False)
    return Port()


@pytest.fixture(scope="session")
def ref():
    from oracle.oracle import Ref

    if not Ref.available():
        pytest.skip("reference sources not compiled here (oracle/_ref)")
    return Ref()


@pytest.fixture(scope="session")
def lib():
    from c2a_gb300 import api, build

    build.build()
    return api.load()


@pytest.fixture(scope="session")
def gpu_ctx(lib):
    import torch
    from c2a_gb300 import api

    if not torch.cuda.is_available():
        pytest.fail("GPU test on a machine without a CUDA device")
    ctx = api.Context(0)
    yield ctx
    ctx.close()
