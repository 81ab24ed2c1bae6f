import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "nnpp-mg-implant-corrosion-3d_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")

if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def load_package():
    """The product package (its directory name is not a Python identifier)."""
    if "nnpp_gb300" in sys.modules:
        return sys.modules["nnpp_gb300"]
    spec = importlib.util.spec_from_file_location(
        "nnpp_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["nnpp_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def nn():
    return load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle


@pytest.fixture(scope="session")
def has_gpu(nn):
    return nn.device_count() > 0
