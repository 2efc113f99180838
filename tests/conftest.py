"""Shared test setup: import paths, the gpu marker, build-on-demand."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "prime-gap_gb300"
for p in (ROOT, PKG, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = ROOT / "tests" / "golden" / "goldens.json"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def built():
    """Build the library, the oracle and the host arithmetic helper (incremental)."""
    import build as pkg_build

    pkg_build.build_lib()
    pkg_build.build_oracle()
    pkg_build.build_arith_host()
    pkg_build.build_tune_host()
    return True


@pytest.fixture(scope="session")
def goldens() -> dict:
    return json.loads(GOLDEN.read_text())


@pytest.fixture(scope="session")
def sieve(built):
    import pgsieve

    s = pgsieve.Sieve(0)
    yield s
    s.close()
