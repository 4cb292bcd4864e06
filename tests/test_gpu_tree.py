"""Octree keys on the GPU with and without the key table (tuning knob 34).

The table (knob 34 = 2: used at any size) replays the first levels of the reference's centre
recursion (BHTree::make's child centres, src/bhtree.cpp:190-196) once per tree build, with the same
FP64 operations, and the key computation searches it with integer comparisons before continuing
the recursion.  The keys, and
therefore the node sets, the particle order and every field after a step, are the same bit for
bit with the table on or off: single runs in 1D, 2D and 3D (with gravity) and batches of runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "ene", "dens", "pres", "sml", "acc", "dene", "alpha", "balsara")


def _cases():
    from sphcode_gb300 import ics
    return {
        "sod_ssph_1d": lambda: (*ics.sod(), None),
        "khi_disph_ac_2d": lambda: (*ics.khi(64, 45), None),
        "evrard_disph_grav_3d": lambda: (*ics.evrard(3000, seed=5), None),
        "ensemble_1d_batch": lambda: ics.ensemble(n_runs=8, n_min=100, n_max=400, seed=3),
        "evrard_3d_batch": lambda: (*ics.evrard(3000, seed=9), [1000, 1200, 800]),
    }


def _run(case, table, prec):
    # table 2: always (the cases are below the default's 2^18-particle threshold)
    from sphcode_gb300 import sphgpu
    p, f, runs = _cases()[case]()
    with sphgpu.GpuSimulation(p, f, precision=prec, runs=runs) as sim:
        sim.set_tuning("autotune", 0)
        sim.set_tuning("key_table", table)
        assert sim.get_tuning("key_table") == table
        sim.initialize()
        sim.step(2)
        out = {name: sim.get(name) for name in FIELDS if name != "balsara" or p.use_balsara}
        out["groups"] = sim.target_groups()[0]
        out["dt"] = np.array([sim.scalar("dt", run=r) for r in range(sim.n_runs)])
    return out


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("case", list(_cases().keys()))
def test_key_table_gives_identical_steps(gpu_lib, case, prec):
    a = _run(case, 2, prec)
    b = _run(case, 0, prec)
    for name in a:
        assert np.array_equal(a[name], b[name]), f"{case} {prec} {name}"
