"""Shared fixtures.  `-m gpu` tests need a CUDA device and the built
libpwmgpu.so; `-m "not gpu"` tests run on CPU only."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpwmgpu.so")


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden_fixtures():
    with open(os.path.join(GOLDEN, "fixtures.json")) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def golden_seeded():
    with open(os.path.join(GOLDEN, "seeded.json")) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def pg():
    import pwm_gb300
    return pwm_gb300


@pytest.fixture(scope="session")
def ctx(pg):
    return pg.default_context()


def words_from_hex(h):
    return np.frombuffer(bytes.fromhex(h), dtype="<u8").astype(np.uint64) if h else np.zeros(0, np.uint64)


def text_from_hex(h):
    return np.frombuffer(bytes.fromhex(h), dtype=np.uint8).copy() if h else np.zeros(0, np.uint8)
