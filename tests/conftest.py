"""Shared test set-up: the `gpu` marker, the package loader and the oracle path.

The package directory is `tealeaf.jl_gb300/` (a dotted name), so it is loaded
by path and registered as the module `tealeaf_gb300`.
"""
import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "tealeaf.jl_gb300"
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(Path(__file__).resolve().parent))
sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))


def load_package():
    if "tealeaf_gb300" in sys.modules:
        return sys.modules["tealeaf_gb300"]
    spec = importlib.util.spec_from_file_location("tealeaf_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["tealeaf_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def tl():
    return load_package()


@pytest.fixture(scope="session")
def built_lib():
    """Builds libtealeaf_gb300.so if needed (nvcc cross-compiles without a GPU)."""
    sys.path.insert(0, str(PKG_DIR))
    import build as tlbuild  # tealeaf.jl_gb300/build.py
    return tlbuild.build()
