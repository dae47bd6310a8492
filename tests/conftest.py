"""Shared fixtures. `-m gpu` tests need a GB300; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def native():
    """Builds (if stale) and loads the product library."""
    from labelpropcuda_gb300 import build as b
    b.build()
    import labelpropcuda_gb300._native as n
    return n.lib()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu(native):
    import labelpropcuda_gb300 as dlp
    if dlp.device_count() < 1:
        pytest.fail("no CUDA device visible for a -m gpu test")
    return dlp
