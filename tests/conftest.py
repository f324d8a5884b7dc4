"""Test configuration: builds the in-tree libraries once per session and
registers the `gpu` marker (tests that need a CUDA device)."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from clustersm_gb300.build import build  # noqa: E402

build()

REF_DATASET = ROOT / "tests" / "golden" / "example"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run with -m gpu)")


@pytest.fixture(scope="session")
def ctx():
    from clustersm_gb300.native import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def example():
    """The reference's example pair (dataset/example_g_01.in, example_q_01.in),
    stored under tests/golden/example/."""
    from clustersm_gb300.native import HostGraph, Query
    g = HostGraph.read(REF_DATASET / "example_g_01.in")
    q = Query.read(REF_DATASET / "example_q_01.in")
    return g, q
