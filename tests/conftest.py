import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def channel_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-channel absolute difference of two BGRA word images, (H, W, 4) int."""
    ab = a.view(np.uint8).reshape(a.shape + (4,)).astype(np.int16)
    bb = b.view(np.uint8).reshape(b.shape + (4,)).astype(np.int16)
    return np.abs(ab - bb)


def assert_parity(got: np.ndarray, want: np.ndarray, max_lsb: int = 1, min_exact: float = 0.999):
    """The raster parity bar: every channel within `max_lsb` and at least `min_exact`
    of pixels bit-exact."""
    assert got.shape == want.shape, (got.shape, want.shape)
    d = channel_diff(got, want)
    worst = int(d.max()) if d.size else 0
    exact = float(np.mean(np.all(d == 0, axis=-1))) if d.size else 1.0
    assert worst <= max_lsb, f"max channel error {worst} LSB > {max_lsb}"
    assert exact >= min_exact, f"only {exact:.5f} of pixels exact"
    return worst, exact


@pytest.fixture(scope="session")
def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
