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
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "grid_rs_vectors.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.lib()
    pyoracle.set_threads(min(16, os.cpu_count() or 1), all_loops=True)
    return pyoracle


@pytest.fixture(scope="session")
def pg():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    import panopaea_gb300

    panopaea_gb300.load()
    return panopaea_gb300


def rng(seed):
    return np.random.default_rng(seed)


def seed_of(*args):
    """Deterministic seed from a test's parameters (str hashing is salted)."""
    import zlib

    return zlib.crc32(repr(args).encode())
