"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libpgx")


@pytest.fixture(scope="session")
def oracle():
    from oracle.ffi import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.ffi import Reference, reference_available
    if not reference_available():
        pytest.skip("reference sources not available on this machine")
    return Reference()


@pytest.fixture(scope="session")
def pgx_lib():
    from pathguidingdissertation_gb300 import build
    build.build()
    from pathguidingdissertation_gb300 import abi
    return abi.load()


@pytest.fixture()
def ctx(pgx_lib):
    from pathguidingdissertation_gb300.api import Context
    c = Context(0)
    yield c
    c.close()
