"""Shared test setup: the `gpu` marker, the oracle and the built library."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as fp:
        g = json.load(fp)
    arrays = dict(np.load(os.path.join(GOLDEN_DIR, "golden_J.npz")))
    return g, arrays


@pytest.fixture(scope="session")
def bflib():
    """The built C-ABI library (compiled on first use if stale)."""
    from beamforming_gb300 import build

    build.build()
    import beamforming_gb300 as bf

    bf.lib()
    return bf


@pytest.fixture(scope="session")
def cuda(bflib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
