"""The allocation-free energy/momentum entry point (sphgpu_energy_noalloc).

It serves callers that cannot allocate device memory where they need the sums, such as a host
that reserves all device memory up front or a loop that must not stall the device.  The
test calls it through the C-ABI on device arrays the test owns, twice in a row, and compares both
results with the context-based sphgpu_energy on the same state (1e-12 relative, the FP64
tolerance of these sums: only the summation order differs).  It also checks that a particle
count beyond the fixed scratch capacity is refused before any device work.

The file name sorts last so that a run stopping at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("case", ["evrard", "khi"])
def test_energy_noalloc_matches_context_sums(gpu_lib, case):
    import torch
    from sphcode_gb300 import ics, sphgpu
    p, f = ics.evrard(3000, seed=5) if case == "evrard" else ics.khi(64, 45)
    with sphgpu.GpuSimulation(p, f, precision="fp64") as sim:
        sim.initialize()
        sim.step(2)
        want = sim.energy()
        fields = {k: torch.from_numpy(np.ascontiguousarray(sim.get(k))).cuda()
                  for k in ("mass", "vel", "ene", "phi")}
    n, dim = int(fields["mass"].shape[0]), p.dim
    lib = sphgpu.library()
    stream = torch.cuda.current_stream()
    results = []
    for _ in range(2):
        out = torch.full((4 + dim,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.sphgpu_energy_noalloc(dim, n, fields["mass"].data_ptr(), fields["vel"].data_ptr(),
                                       fields["ene"].data_ptr(),
                                       fields["phi"].data_ptr() if p.use_gravity else None,
                                       out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.sphgpu_last_error(None)
        torch.cuda.synchronize()
        results.append(out.cpu().numpy())
    for got in results:
        assert np.all(np.isfinite(got))
        # momentum components can be ~0: compare them against the kinetic-energy scale
        assert _rel(got[:4], want[:4]) <= TOL, (got, want)
        scale = np.sqrt(2.0 * want[0] * float(np.sum(f["mass"]))) + 1e-300
        assert float(np.max(np.abs(got[4:] - want[4:]))) <= TOL * scale, (got, want)
    assert np.array_equal(results[0], results[1])


def test_energy_noalloc_rejects_oversize(gpu_lib):
    from sphcode_gb300 import sphgpu
    lib = sphgpu.library()
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    rc = lib.sphgpu_energy_noalloc(3, 33554432 + 1, dummy, dummy, dummy, None, dummy, None)
    assert rc == 4
    assert b"exceeds the fixed scratch capacity" in lib.sphgpu_last_error(None)
    assert lib.sphgpu_energy_noalloc(3, 0, dummy, dummy, dummy, None, dummy, None) == 1
