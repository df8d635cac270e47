"""Shared pytest setup: the `gpu` marker, import paths, golden-fixture loader."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "xpbd-fem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libxfem.so")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_args(name):
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)[name]


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle
