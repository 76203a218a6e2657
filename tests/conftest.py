import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "x86-simd-sort_gb300")
for p in (ROOT, PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def _load_build():
    spec = importlib.util.spec_from_file_location("xss_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def xss():
    """The product library (libxss_gb300.so via pyxss), built in-tree if stale."""
    _load_build().build()
    import pyxss
    pyxss.lib()
    return pyxss


@pytest.fixture(scope="session")
def oracle():
    """CPU oracle (test infrastructure): restatement of the reference's scalar path."""
    from oracle import pyoracle
    return pyoracle.oracle()


@pytest.fixture(scope="session")
def cuda(xss):
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("GPU test collected on a host without a CUDA device")
    torch.cuda.init()
    return torch
