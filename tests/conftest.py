"""Shared fixtures.  `gpu`-marked tests need a CUDA device and the built library;
everything else runs on the CPU (the library's host-only entry points and the
CPU oracle)."""
from __future__ import annotations

import importlib
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def pq():
    import __graft_entry__ as ge

    ge.build()
    return importlib.import_module("prism-q_gb300")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    return np.load(ROOT / "tests" / "golden" / "neighbor_golden.npz")


@pytest.fixture(scope="session")
def gpu(pq):
    if pq.device_count() < 1:
        raise RuntimeError("gpu-marked test ran without a CUDA device")
    return pq


@pytest.fixture(scope="session")
def ala250(pq):
    return pq.Topology.polyala(1, 250, seed=1)


@pytest.fixture(scope="session")
def ala40(pq):
    return pq.Topology.polyala(1, 40, seed=11)


def rel_rms(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))
