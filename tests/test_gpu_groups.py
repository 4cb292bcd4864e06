"""Target groups of the pair kernels on the GPU: both formation rules (knob 30) partition every
run's particles into groups of at most 32 x group_warps, and the pair kernels give the oracle's
results with either rule (through the C-ABI)."""
import numpy as np
import pytest

from conftest import assert_counts_match, rel_err

pytestmark = pytest.mark.gpu


def _cases():
    from sphcode_gb300 import ics
    return {
        "khi_disph_ac_2d": lambda: ics.khi(64, 45),
        "evrard_disph_grav_3d": lambda: ics.evrard(4000, seed=7),
        "sod_ssph_1d": lambda: ics.sod(),
    }


@pytest.mark.parametrize("rule", [1, 0])
@pytest.mark.parametrize("warps", [1, 2, 4])
@pytest.mark.parametrize("case", list(_cases().keys()))
def test_groups_partition_runs(gpu_lib, case, warps, rule):
    from sphcode_gb300 import sphgpu
    p, f = _cases()[case]()
    with sphgpu.GpuSimulation(p, f, precision="fp32") as sim:
        sim.set_tuning("group_warps", warps)
        sim.set_tuning("group_rule", rule)
        sim.initialize()
        sim.step(1)
        g, ng = sim.target_groups()
        assert ng > 0 and g.min() >= 0 and g.max() == ng - 1
        sizes = np.bincount(g, minlength=ng)
        assert sizes.min() >= 1 and sizes.max() <= 32 * warps


def test_batch_groups_stay_in_their_run(gpu_lib):
    from sphcode_gb300 import ics, sphgpu
    # runs smaller and larger than a group, back to back
    p, f, counts = ics.ensemble(n_runs=8, n_min=20, n_max=300, seed=5)
    with sphgpu.GpuSimulation(p, f, precision="fp32", runs=counts) as sim:
        sim.set_tuning("group_warps", 4)
        sim.initialize()
        sim.step(1)
        g, ng = sim.target_groups()
        run_of = np.repeat(np.arange(len(counts)), counts)
        for k in range(ng):
            assert len(set(run_of[g == k])) == 1
        assert np.bincount(g).max() <= 128


@pytest.mark.parametrize("knob", [("group_rule", 0), ("prewalk", 1), ("prewalk", 3), ("gravity_items", 0)])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("case", ["khi_disph_ac_2d", "evrard_disph_grav_3d"])
def test_alternative_group_setups_parity(gpu_lib, case, prec, knob):
    """The former group rule (fixed chunks split once), the group plans (a walk kernel ahead of
    the first pass, for FluidForce or both stages) and the gravity walk over the pair groups' pieces
    instead of fixed 32-particle chunks stay selectable and match the oracle."""
    from oracle import pyoracle
    from sphcode_gb300 import sphgpu
    from test_gpu_parity import FP32_TOL, FP64_TOL, _fields
    p, f = _cases()[case]()
    ref = pyoracle.OracleSim(p, f, kind="port")
    ref.initialize()
    ref.step()
    with sphgpu.GpuSimulation(p, f, precision=prec) as sim:
        sim.set_tuning(*knob)
        sim.initialize()
        sim.step(1)
        for name in _fields(p):
            e = rel_err(sim.get(name), ref.get(name))
            tol = FP64_TOL if prec == "fp64" else FP32_TOL.get(name, 1e-4)
            assert e <= tol, f"{case} {prec} {name}: {e:.3e}"
        assert_counts_match(sim.get("neighbor"), ref.get("neighbor"), ref.get("pos"), ref.get("sml"),
                            p, 1e-12 if prec == "fp64" else 2e-5)
