"""Shared test configuration: the ``gpu`` marker and helpers used by the parity tests."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


def rel_err(a, b) -> float:
    """max |a - b| / max |b| over all components (0 when both vanish)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = float(np.max(np.abs(a - b))) if a.size else 0.0
    s = float(np.max(np.abs(b))) if b.size else 0.0
    if s == 0.0:
        return d
    return d / s


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library on a machine with a GPU (the product path; no fallback)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()
    from sphcode_gb300 import sphgpu
    return sphgpu.library()
