import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "dcu-winograd-conv2d_gb300")
for path in (ROOT, os.path.join(ROOT, "oracle")):
    if path not in sys.path:
        sys.path.insert(0, path)


def load_wgconv():
    """The operator's Python mirror (package directory name has hyphens)."""
    if "wgconv" in sys.modules:
        return sys.modules["wgconv"]
    spec = importlib.util.spec_from_file_location("wgconv", os.path.join(PKG_DIR, "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["wgconv"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def wg():
    mod = load_wgconv()
    mod.build()  # incremental: a no-op when nothing changed
    mod.lib()
    return mod
