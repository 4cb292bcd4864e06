"""The C++ Module drop-ins (sphcode_gb300/cxx/gpu_modules.cpp) inside the reference's own code.

oracle/build_ref.sh links the GPU modules sph::gpu::{PreInteraction, FluidForce, GravityForce}
with the reference's unmodified Simulation, BHTree, TimeStep and exhaustive-search sources and
the harness that restates Solver::initialize / integrate / predict / correct
(src/solver.cpp:353-474); the harness plugs the GPU modules in at the module switch of
Solver::initialize (src/solver.cpp:359-370).  Each case drives Module::calculation() in Solver
order through that build and through the build with the reference's own modules, from the same
inputs, and compares the particle fields after initialize and after three steps:

  GPU modules in FP64     : every field within 1e-9 relative of the reference modules;
  GPU modules in FP32-pair: per field FP32_TOL of test_gpu_parity.py.

Neighbour counts are compared with the r = h tie rule of the other parity tests.  The wall time
of one Solver::integrate step through the per-module path (an AoS upload and download around
every calculation()) is printed beside the reference's.
"""
import time

import numpy as np
import pytest

from conftest import assert_counts_match, rel_err
from test_gpu_parity import FP32_TOL, FP64_TOL, _cases, _fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(gpu_lib):
    from oracle import pyoracle
    if not pyoracle.gpu_modules_available():
        pytest.skip("the reference sources were not available to oracle/build_ref.sh")
    return True


@pytest.mark.parametrize("prec", [1, 0], ids=["fp64", "fp32"])
@pytest.mark.parametrize("case", list(_cases().keys()))
def test_modules_in_reference_solver(built, case, prec):
    from oracle import pyoracle
    p, f = _cases()[case]()
    ref = pyoracle.OracleSim(p, f, kind="ref", flavor="strict")
    gm = pyoracle.OracleSim(p, f, kind="gpumod", gpu_precision=prec)
    name = "fp64" if prec == 1 else "fp32"
    for stage in ("initialize", "3 steps"):
        if stage == "initialize":
            ref.initialize()
            gm.initialize()
        else:
            t0 = time.perf_counter()
            for _ in range(3):
                ref.step()
            t_ref = (time.perf_counter() - t0) / 3
            t0 = time.perf_counter()
            for _ in range(3):
                gm.step()
            t_gm = (time.perf_counter() - t0) / 3
            print(f"\n[cxx modules] {case} {name}: one step {t_gm * 1e3:.2f} ms through the GPU modules, "
                  f"{t_ref * 1e3:.2f} ms through the reference modules ({ref.n} particles)")
        names = _fields(p) + (["pos", "vel", "ene"] if stage != "initialize" else [])
        for n_ in names:
            e = rel_err(gm.get(n_), ref.get(n_))
            tol = FP64_TOL if prec == 1 else FP32_TOL.get(n_, 1e-4)
            assert e <= tol, f"{case} {name} {stage}: {n_} rel err {e:.3e} > {tol:.1e}"
        assert_counts_match(gm.get("neighbor"), ref.get("neighbor"), ref.get("pos"), ref.get("sml"), p,
                            1e-12 if prec == 1 else 2e-5)
        assert abs(gm.scalar("time") - ref.scalar("time")) <= (1e-12 if prec == 1 else 1e-4) * max(ref.scalar("time"), 1e-300)
    gm.close()
    ref.close()


def test_module_error_becomes_sph_exception(built):
    """A status the library returns surfaces as the reference's SPHException (THROW_ERROR) with
    the library's message: here a 3D tree deeper than the 64-bit octree keys hold, which the
    library refuses when the first calculation() creates its context."""
    from oracle import pyoracle
    from sphcode_gb300 import ics
    p, f = ics.evrard(500, seed=3)
    p.max_level = 30
    gm = pyoracle.OracleSim(p, f, kind="gpumod", gpu_precision=1)
    with pytest.raises(RuntimeError) as e:
        gm.initialize()
    assert "sphgpu create" in str(e.value) and "maxTreeLevel" in str(e.value)
    gm.close()
