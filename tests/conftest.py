import importlib.util
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "flame-fractal-renderer_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")

for p in (PKG, ORACLE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def built():
    """Build the library and the oracle once per session (no-op if fresh)."""
    import __graft_entry__ as ge
    ge.build()
    return ge


@pytest.fixture(scope="session")
def ffr(built):
    import ffr as mod
    mod.load_library()
    return mod


@pytest.fixture(scope="session")
def fo():
    import flame_oracle as mod
    mod.build()
    return mod


@pytest.fixture(scope="session")
def flames():
    import flames as mod
    return mod


def golden_manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def golden_flame_text(name):
    with open(os.path.join(GOLDEN, "flames", name + ".json")) as f:
        return f.read()
