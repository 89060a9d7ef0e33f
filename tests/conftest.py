"""Shared test setup.

Markers: ``gpu`` tests need a CUDA device and the in-tree libps_gpu.so; all
others run on CPU.  The CPU oracle (oracle/) is test infrastructure and is
built on demand.
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "plaquette-simulator_gb300", "python"))
sys.path.insert(0, os.path.join(ROOT, "plaquette-simulator_gb300"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the in-tree CUDA library")


@pytest.fixture(scope="session")
def O():
    import oracle
    oracle.build(ref=True)
    return oracle


@pytest.fixture(scope="session")
def kat():
    with open(os.path.join(GOLDEN, "reference_kat.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ref_runs():
    with open(os.path.join(GOLDEN, "reference_runs.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ref_circuits():
    """The reference's benchmark circuits with the reference's own outputs
    (make_golden.py: benchmarks/circuits.tar.gz run on oracle/_ref)."""
    with open(os.path.join(GOLDEN, "reference_circuits.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; skips without a GPU."""
    import build as psbuild
    psbuild.build()
    import torch  # noqa: F401  (device presence check only)
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from plaquette_simulator import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def ps(gpu_lib):
    import plaquette_simulator
    return plaquette_simulator


def tableau_equal(a, b):
    return all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))
