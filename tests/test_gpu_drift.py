"""Energy and momentum over full runs, GPU against the oracle.

Each reduced-size workload runs from Solver::initialize to its endTime (the reference's loop,
src/solver.cpp:417-429: integrate while time < endTime) on the C oracle (strict FP64) and on the
GPU in both arithmetic forms, for the oracle's number of steps.  Compared: the relative drift of
the total energy E = E_k + E_t + E_p (src/output.cpp:66-90), dE = (E_end - E_0) / |E_0|, and the
final momentum sum P = sum m v.

Tolerances (stated per form; the runs are long enough for rounding differences to grow, so the
bounds are on the drift, not on the final states):
  FP64 form      : |dE_gpu - dE_oracle| <= 0.02 |dE_oracle| + 1e-9; |P_gpu - P_oracle| <= 0.02 |P_oracle|
                   + 1e-9 P_scale, with P_scale = sum m |v| of the oracle's final state.
  FP32-pair form : |dE_gpu - dE_oracle| <= 0.25 |dE_oracle| + 2e-6; |P_gpu - P_oracle| <= 0.5 |P_oracle|
                   + 2e-5 P_scale (per-particle pair sums in FP32 are not exactly antisymmetric, and
                   the Barnes-Hut momentum error of the Evrard run depends on the trajectory).
  Start energy   : 1e-9 (FP64) / 1e-6 (FP32-pair) relative.  Time after the oracle's step count:
                   1e-6 (FP64) / 5e-3 (FP32-pair: the time steps follow the trajectory, and the
                   Kelvin-Helmholtz and Evrard runs amplify rounding differences).

Measured on a GB300 (FP64 form, oracle): Sod dE/E -3.007246e-06 / -3.007246e-06, Gresho
7.746093e-05 / 7.746093e-05, KHI 4.795416e-04 / 4.795416e-04, Evrard -1.253122e-02 /
-1.253122e-02; FP32-pair form -3.0127e-06, 7.7431e-05, 4.7423e-04, -1.2448e-02.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": (0.02, 1e-9, 0.02, 1e-9), "fp32": (0.25, 2e-6, 0.5, 2e-5)}


def _cases():
    from sphcode_gb300 import ics
    return {
        "sod_900": (lambda: ics.sod(), 0.2),
        "gresho_32x32": (lambda: ics.gresho(32), 1.0),
        "khi_64x45": (lambda: ics.khi(64, 45), 2.0),
        "evrard_4000": (lambda: ics.evrard(4000, seed=7), 3.0),
    }


_ORACLE = {}


def _oracle_run(case):
    """Oracle energies at the start and the end, final momentum scale and the step count."""
    if case in _ORACLE:
        return _ORACLE[case]
    from oracle import pyoracle
    make, end = _cases()[case]
    p, f = make()
    ref = pyoracle.OracleSim(p, f, kind="port")
    ref.initialize()
    e0 = ref.energy()
    steps = 0
    while ref.scalar("time") < end:
        ref.step()
        steps += 1
    e1 = ref.energy()
    v = ref.get("vel").reshape(ref.n, -1)
    pscale = float(np.sum(ref.get("mass") * np.sqrt((v * v).sum(1))))
    _ORACLE[case] = (e0, e1, steps, ref.scalar("time"), pscale)
    ref.close()
    return _ORACLE[case]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("case", list(_cases().keys()))
def test_energy_and_momentum_drift(gpu_lib, case, prec):
    from sphcode_gb300 import sphgpu
    e0r, e1r, steps, t_end, pscale = _oracle_run(case)
    make, _ = _cases()[case]
    p, f = make()
    D = p.dim
    with sphgpu.GpuSimulation(p, f, precision=prec) as sim:
        sim.initialize()
        e0 = sim.energy()
        sim.step(steps)
        e1 = sim.energy()
        t = sim.scalar("time")
    drift_ref = (e1r[3] - e0r[3]) / abs(e0r[3])
    drift = (e1[3] - e0[3]) / abs(e0[3])
    p_ref, p_gpu = e1r[4:4 + D], e1[4:4 + D]
    dp = float(np.max(np.abs(p_gpu - p_ref)))
    print(f"\n[drift] {case} {prec}: steps {steps} t {t:.6f} (oracle {t_end:.6f}) "
          f"dE/E gpu {drift:.6e} oracle {drift_ref:.6e} | P gpu {p_gpu.tolist()} oracle {p_ref.tolist()} "
          f"P_scale {pscale:.6e}")
    a_e, b_e, a_p, b_p = TOL[prec]
    assert abs(e0[3] - e0r[3]) <= (1e-9 if prec == "fp64" else 1e-6) * abs(e0r[3]), (e0, e0r)
    assert abs(t - t_end) <= (1e-6 if prec == "fp64" else 5e-3) * t_end
    assert abs(drift - drift_ref) <= a_e * abs(drift_ref) + b_e, (drift, drift_ref)
    assert dp <= a_p * float(np.max(np.abs(p_ref))) + b_p * pscale, (p_gpu, p_ref, pscale)
