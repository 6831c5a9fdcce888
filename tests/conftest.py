"""Shared fixtures. Tests marked `gpu` need a CUDA device and call the CUDA
path through the C ABI; everything else runs on the CPU (oracle, host logic,
library loading)."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG = "neural-mixture-guiding_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; exercises the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: long CPU-side check, run with --runslow")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    _mark_slow(config, items)
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def nmg():
    return importlib.import_module(PKG)


@pytest.fixture(scope="session")
def synth():
    return importlib.import_module(PKG + ".synth")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    return O


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "mixture_golden.npz")))


def pytest_addoption(parser):
    parser.addoption("--runslow", action="store_true", default=False, help="run tests marked slow")


def _mark_slow(config, items):
    if config.getoption("--runslow"):
        return
    import os
    if os.environ.get("NMG_RUN_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow CPU test (use --runslow)")
    for it in items:
        if "slow" in it.keywords:
            it.add_marker(skip)
