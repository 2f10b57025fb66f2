"""Shared test configuration.

Markers: ``gpu`` -- needs a GB300 (sm_103a) and the built CUDA library; everything else runs on CPU.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built sm_103a library")


@pytest.fixture(scope="session")
def golden_dir():
    return ROOT / "tests" / "golden"
