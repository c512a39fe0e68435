"""Shared fixtures of the test suite.

Tests marked ``gpu`` need a CUDA device (run with ``-m gpu`` on a GB300);
everything else runs on the CPU (``-m "not gpu"``). The native library and the
oracle are built in-tree on first use.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """The product library, built if missing."""
    from onesolver_gb300 import build
    build.build_library()
    import onesolver_gb300 as osg
    osg.lib()
    return osg


@pytest.fixture(scope="session")
def orc():
    """The oracle (CPU restatement of the reference), built if missing."""
    import oracle
    oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def golden_exhaustive():
    return json.loads((GOLDEN / "exhaustive_golden.json").read_text())


@pytest.fixture(scope="session")
def golden_io():
    return json.loads((GOLDEN / "io_golden.json").read_text())


@pytest.fixture(scope="session")
def golden_chimera():
    return json.loads((GOLDEN / "chimera_golden.json").read_text())


@pytest.fixture(scope="session")
def ctx(native):
    c = native.Context(0)
    yield c
    c.close()
