"""Test setup: registers the `gpu` marker and makes sure the in-tree library
and the CPU oracle are built before any test imports them."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _ensure_built() -> None:
    lib = os.path.join(ROOT, "kclistpp_gb300", "libkclpp.so")
    spec = importlib.util.spec_from_file_location("_kclpp_build", os.path.join(ROOT, "kclistpp_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()  # incremental: only stale objects are rebuilt
    assert os.path.exists(lib)
    from oracle import oracle

    oracle.build()


_ensure_built()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def gpu_available() -> bool:
    try:
        import kclistpp_gb300 as K

        K.Context(0).close()
        return True
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    import kclistpp_gb300 as K

    c = K.Context(0)
    yield c
    c.close()
