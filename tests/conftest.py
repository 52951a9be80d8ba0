"""Shared test setup: the `gpu` marker, repository paths and golden fixtures."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_arrays():
    return np.load(os.path.join(GOLDEN, "mapping_cases.npz"))


@pytest.fixture(scope="session")
def parser_cases():
    with open(os.path.join(GOLDEN, "parser_cases.json")) as f:
        return json.load(f)


def case_names():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return sorted(json.load(f)["cases"].keys())
