"""Shared pytest setup.

Markers:
  gpu  -- needs a CUDA device and the built libgbpoly.so; run with `-m gpu`.
Everything else runs on a CPU-only machine.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "sycl-bench_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


@pytest.fixture(scope="session")
def ctx():
    import gbpoly

    c = gbpoly.Context(0)
    yield c
    c.close()
