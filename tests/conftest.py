"""pytest configuration: the `gpu` marker, and in-tree builds of the native
library and the oracles when they are missing (cheap no-ops otherwise)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from pyrsgm_gb300 import build as libbuild
    libbuild.build()
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_oracle", os.path.join(ROOT, "oracle", "build_oracle.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    m.build_oracle()
    try:
        m.build_harness()
        m.build_ref_fatbins()
    except RuntimeError:
        pass
    yield


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
