"""Shared fixtures.  GPU tests carry the ``gpu`` marker; everything else runs
on a CPU-only machine (the engine library is still built and loaded there,
but no compute call is made without a GPU)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU; run with -m gpu")


@pytest.fixture(scope="session")
def enginelib():
    """The engine's shared library, built in-tree if it is missing."""
    from bioshell_gb300 import _build, lib
    if not os.path.exists(lib.LIB_PATH):
        _build.build()
    return lib.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def engine(enginelib):
    from bioshell_gb300.crmsd import Engine
    eng = Engine(0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def golden_small():
    return np.load(os.path.join(GOLDEN, "decoys_small.npz"))


@pytest.fixture(scope="session")
def golden_2jqb():
    return np.load(os.path.join(GOLDEN, "models_2jqb.npz"))
