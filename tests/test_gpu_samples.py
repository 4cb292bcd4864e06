"""The reference's six samples (src/sample/*.cpp initial conditions with the parameters of their
sample/*/*.json files) on the GPU against the oracle.

The parameters are those the reader gives for each sample file (checked against the files in
tests/test_samples.py); they are built here from that table so that nothing reads the reference
at run time.  Each sample runs Solver::initialize and three Solver::integrate steps on the GPU in
both forms and on the C oracle; tolerances as in test_gpu_parity.py (FP64 1e-9 on every field,
FP32-pair FP32_TOL; neighbour counts equal except at r = h ties).
"""
import pytest

from conftest import assert_counts_match, rel_err
from test_gpu_parity import FP32_TOL, FP64_TOL, _fields
from test_samples import EXPECTED

pytestmark = pytest.mark.gpu


def _params(name):
    from sphcode_gb300.params import SPHParameters
    want = dict(EXPECTED[name])
    D = want["dim"]
    sample_n = want.pop("sample_n")
    for k in ("range_min", "range_max"):
        if k in want:
            want[k] = list(want[k]) + [0.0] * (3 - D)
    p = SPHParameters(**want)
    p.sample, p.sample_n = name, sample_n
    return p


def _initial(name, p):
    from sphcode_gb300 import ics
    N, g = p.sample_n, p.gamma
    return {"shock_tube": lambda: ics.sample_shock_tube(N, g),
            "khi": lambda: ics.sample_khi(N, g),
            "evrard": lambda: ics.sample_evrard(N, g, p.g_constant),
            "gresho_chan_vortex": lambda: ics.sample_gresho_chan_vortex(N, g),
            "hydrostatic": lambda: ics.sample_hydrostatic(N, g),
            "pairing_instability": lambda: ics.sample_pairing_instability(N, g)}[name]()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("name", list(EXPECTED))
def test_reference_sample(gpu_lib, name, prec):
    from oracle import pyoracle
    from sphcode_gb300 import sphgpu
    p = _params(name)
    f = _initial(name, p)
    ref = pyoracle.OracleSim(p, f, kind="port")
    ref.initialize()
    with sphgpu.GpuSimulation(p, f, precision=prec) as sim:
        sim.initialize()
        for stage in ("initialize", "3 steps"):
            if stage != "initialize":
                for _ in range(3):
                    ref.step()
                sim.step(3)
            names = _fields(p) + (["pos", "vel", "ene"] if stage != "initialize" else [])
            for n_ in names:
                e = rel_err(sim.get(n_), ref.get(n_))
                tol = FP64_TOL if prec == "fp64" else FP32_TOL.get(n_, 1e-4)
                assert e <= tol, f"{name} {prec} {stage}: {n_} rel err {e:.3e} > {tol:.1e}"
            assert_counts_match(sim.get("neighbor"), ref.get("neighbor"), ref.get("pos"), ref.get("sml"),
                                p, 1e-12 if prec == "fp64" else 2e-5)
    ref.close()
