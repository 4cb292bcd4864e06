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


def reference_root():
    """A directory holding the reference's sample/ parameter files: $SPHCODE_REFERENCE, or the
    source snapshot the oracle recipe keeps in oracle/_ref/snapshot; None when neither exists."""
    for cand in (os.environ.get("SPHCODE_REFERENCE"), os.path.join(ROOT, "oracle", "_ref", "snapshot")):
        if cand and os.path.isdir(os.path.join(cand, "sample")):
            return cand
    return None


def knife_edge(pos, h, i, periodic=None, rel=1e-12):
    """True if some particle lies within rel * h[i] of the distance h[i] from particle i (then
    the last bits of h decide whether it counts as a neighbour).  periodic = (lo, hi) arrays."""
    pos = np.asarray(pos, dtype=np.float64).reshape(len(h), -1)
    d = pos - pos[i]
    if periodic is not None:
        L = np.asarray(periodic[1]) - np.asarray(periodic[0])
        L = L[:d.shape[1]]
        d = np.where(np.abs(d + L) < np.abs(d), d + L, d)
        d = np.where(np.abs(d - L) < np.abs(d), d - L, d)
    r = np.sqrt((d * d).sum(1))
    return bool(np.any(np.abs(r - h[i]) <= rel * h[i]))


def assert_counts_match(nb_gpu, nb_ref, pos, h_ref, params, rel):
    """Neighbour counts equal, except at knife-edge particles (see knife_edge)."""
    bad = np.nonzero(np.asarray(nb_gpu) != np.asarray(nb_ref))[0]
    per = (params.range_min, params.range_max) if params.periodic else None
    not_edge = [int(i) for i in bad if not knife_edge(pos, h_ref, int(i), per, rel)]
    assert not not_edge, f"neighbour counts differ away from r = h ties at {not_edge[:10]} " \
                         f"({len(not_edge)} of {len(bad)} mismatches)"
    return len(bad)
