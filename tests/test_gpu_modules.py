"""The reference-shaped host API (sphcode_gb300/modules.py): Solver.integrate through the Module
subclasses equals the device step loop, and Solver.run writes the reference's output formats."""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_module_path_equals_step_graph(gpu_lib):
    from sphcode_gb300 import ics, modules, sphgpu
    p, f = ics.gresho(32)
    s = modules.Solver(p, f, precision="fp64")
    s.initialize()
    for _ in range(3):
        s.integrate()
    with sphgpu.GpuSimulation(p, f, precision="fp64") as g:
        g.initialize()
        g.step(3)
        # the step graph forms the predicted sound speed in the Pre/Fluid mirrors, the module path
        # stores it in predict: the same FP64 expression, so the same forces and the same state
        for k in ("pos", "vel", "ene", "dens", "acc", "dene", "sound", "alpha", "pres"):
            assert rel_err(s.sim.gpu.get(k), g.get(k)) <= 1e-13, k
        assert s.sim.get_time() == pytest.approx(g.scalar("time"), rel=1e-15)
    s.close()


def test_run_writes_reference_formats(gpu_lib, tmp_path):
    from oracle import pyoracle
    from sphcode_gb300 import ics, modules
    p, f = ics.sod(200, 25)
    p.end_time = 0.02
    p.output_time = 0.01
    p.energy_time = 0.005
    s = modules.Solver(p, f, precision="fp64", output_dir=str(tmp_path))
    steps = s.run()
    s.close()
    assert steps > 0
    dumps = sorted(x for x in os.listdir(tmp_path) if x.endswith(".dat") and x != "energy.dat")
    assert dumps[0] == "00000.dat" and len(dumps) >= 2
    rows = np.loadtxt(tmp_path / dumps[0])
    assert rows.shape == (225, 3 * 1 + 9)          # pos vel acc + 9 scalar columns in 1D
    assert np.array_equal(rows[:, 3 + 5], np.arange(225))   # id column
    e = np.loadtxt(tmp_path / "energy.dat")
    assert e.shape[1] == 5
    # the first energy line is the initial state: compare with the oracle
    ref = pyoracle.OracleSim(p, f, kind="port")
    ref.initialize()
    assert rel_err(e[0, 1:], ref.energy()[:4]) <= 1e-12
