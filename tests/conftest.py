"""pytest configuration: the `gpu` marker and loaders for the package
(`millepede-ii_gb300/`, loaded by path) and the oracle binding."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "millepede-ii_gb300")
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def load_pkg_module(name):
    full = "millepede_ii_gb300_" + name
    if full in sys.modules:
        return sys.modules[full]
    spec = importlib.util.spec_from_file_location(full, os.path.join(PKG, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[full] = mod
    spec.loader.exec_module(mod)
    return mod


def _ensure_built():
    mp = load_pkg_module("mpgpu")
    orc = os.path.join(ROOT, "oracle", "_build", "libmpref.so")
    if not (os.path.exists(mp.LIBPATH) and os.path.exists(orc)):
        b = load_pkg_module("build")
        b.build_all()


@pytest.fixture(scope="session")
def mp():
    _ensure_built()
    return load_pkg_module("mpgpu")


@pytest.fixture(scope="session")
def orc():
    _ensure_built()
    import oracle_ref
    return oracle_ref
