import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_DIR = os.path.join(ROOT, "imagequilting.jl_gb300")


def load_package():
    """Import the package directory `imagequilting.jl_gb300` under the module name `iqgpu`."""
    if "iqgpu" in sys.modules:
        return sys.modules["iqgpu"]
    spec = importlib.util.spec_from_file_location(
        "iqgpu", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["iqgpu"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def iq():
    return load_package()
