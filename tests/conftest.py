"""Shared pytest setup: the `gpu` marker, the package under test and the CPU oracle."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import __graft_entry__  # noqa: E402

dpg = __graft_entry__.load_package()  # registers sys.modules["smdp_gb300"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: full-size workloads (minutes)")


def load_golden(name: str) -> dict:
    return json.loads((GOLDEN / name).read_text())


@pytest.fixture(scope="session")
def lib():
    return dpg.load_library()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.oracle_lib()
    return oracle


@pytest.fixture(scope="session")
def ctx():
    c = dpg.Context(0)
    yield c
    c.close()
