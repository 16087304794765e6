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
def hd_golden():
    """The 1080p fixtures (tests/golden/me_1080p.npz, made by the compiled
    reference) and the benchmark-sequence frames they were made from,
    regenerated here and checked against the stored SHA-256."""
    import hashlib

    from imagecodingutils_gb300 import synth
    g = dict(np.load(os.path.join(GOLDEN, "me_1080p.npz")))
    seed, w, h, mr, *pairs = (int(v) for v in g["meta"])
    fr = synth.pan_sequence(seed, w, h, max(pairs) + 2)
    digest = hashlib.sha256(b"".join(np.ascontiguousarray(f, np.int16).tobytes() for f in fr)).digest()
    assert digest == g["frames_sha256"].tobytes(), "the synthetic generator no longer makes the fixtures' frames"
    return {"g": g, "frames": fr, "w": w, "h": h, "motion_range": mr, "pairs": pairs}


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
