"""Shared pytest setup.

GPU tests carry ``@pytest.mark.gpu``; ``-m "not gpu"`` runs the CPU suite
(oracle vs. the reference's known-answer tests, host logic, library exports).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "itensors.jl_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def nd():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    import ndtensors_gb300 as nd
    nd.load()
    return nd
