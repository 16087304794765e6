"""Shared pytest set-up: the `gpu` marker, import paths and the CPU oracle.

Tests marked `gpu` need a GB300 and the built CUDA library; everything else
runs on any host (the oracle, the golden fixtures, the C ABI's exports).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build(with_reference=False)
    return oracle.Oracle()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name)))
    return load


@pytest.fixture(scope="session")
def vpp():
    import imagecodingutils_gb300 as vpp
    from imagecodingutils_gb300 import build
    build.build()
    vpp.load()
    return vpp


@pytest.fixture(scope="session")
def ctx(vpp):
    return vpp.get_context()
