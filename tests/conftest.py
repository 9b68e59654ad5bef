"""pytest configuration: the `gpu` marker, the package loader and the oracle path."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "gradientrobustmultiphysics.jl_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def load_package():
    """Import the package directory (its name holds a dot) as `grmp_gb300`."""
    if "grmp_gb300" in sys.modules:
        return sys.modules["grmp_gb300"]
    spec = importlib.util.spec_from_file_location("grmp_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["grmp_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the C-ABI library's kernels)")


@pytest.fixture(scope="session")
def G():
    return load_package()


@pytest.fixture(scope="session")
def O():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx(G):
    """A library context on cuda:0 (GPU tests only)."""
    import grmp_gb300.build as b
    b.build()
    c = G.GB300Context(0)
    yield c
    c.close()
