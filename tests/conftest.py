import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "beamcast-gx-v1.0-beta-_gb300")
for p in (PKG_DIR, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU; runs the CUDA path")


@pytest.fixture(scope="session")
def pins():
    with open(os.path.join(ROOT, "tests", "golden", "reference_pins.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def native_lib():
    """The in-tree C-ABI library, built on demand (host compile only; no GPU needed)."""
    import build as native_build
    native_build.build()
    import bcgx
    bcgx.lib()
    return bcgx


@pytest.fixture(scope="session")
def gpu_ctx(native_lib):
    bcgx = native_lib
    ok, why = bcgx.gpu_available()
    assert ok, f"GPU test needs a GB300: {why}"
    ctx = bcgx.Context(0)
    yield ctx
    ctx.close()
