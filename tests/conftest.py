import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "eom-imsrg_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libimsrg_gb300.so")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def load_build_module():
    import importlib.util
    path = os.path.join(ROOT, "eom-imsrg_gb300", "build.py")
    spec = importlib.util.spec_from_file_location("imsrg_gb300_build", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built_lib():
    return load_build_module().build()


@pytest.fixture(scope="session")
def oracles():
    from imsrg_gb300.basis import make_basis
    from oracle.oracle import Oracle
    cache = {}

    def get(emax):
        if emax not in cache:
            cache[emax] = Oracle(make_basis(emax))
        return cache[emax]
    return get


@pytest.fixture(scope="session")
def engines(built_lib):
    from imsrg_gb300 import Engine
    from imsrg_gb300.basis import make_basis
    cache = {}

    def get(emax):
        if emax not in cache:
            cache[emax] = Engine(make_basis(emax), device=0)
        return cache[emax]
    return get
