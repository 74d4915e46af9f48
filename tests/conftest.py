"""Shared test set-up: import paths, the ``gpu`` marker, small helpers."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "level-set-method-code_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblsgb.so")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def port():
    from oracle import Oracle
    return Oracle("port")


@pytest.fixture(scope="session")
def lsgb_mod():
    """The product binding with the CUDA library built (fails loudly if the
    build fails -- there is no fallback)."""
    import __graft_entry__ as ge
    ge.build_library()
    import lsgb
    lsgb.lib()
    return lsgb


@pytest.fixture(scope="session")
def cuda(lsgb_mod):
    if not gpu_available():
        pytest.fail("test marked gpu needs a CUDA device (run with -m 'not gpu' on CPU hosts)")
    import torch
    torch.cuda.init()
    return torch.device("cuda:0")
