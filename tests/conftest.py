"""Test configuration: the `gpu` marker and shared helpers.

CPU tests (`-m "not gpu"`) check the oracle against the golden fixtures and
the library's C ABI without touching a GPU.  GPU tests (`-m gpu`) call the
CUDA library through its C ABI and compare with the oracle.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libtridiag.so")


@pytest.fixture(scope="session")
def golden():
    d = ROOT / "tests" / "golden"
    return {
        "f64": np.load(d / "ref_cpu_f64.npz"),
        "f32": np.load(d / "ref_cpu_f32.npz"),
        "gtsv": np.load(d / "lapack_gtsv.npz"),
        "kat": np.load(d / "kat_laplacian.npz"),
    }


@pytest.fixture(scope="session")
def cuda():
    """torch with a CUDA device; GPU tests fail (not skip) without one."""
    import torch

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch
