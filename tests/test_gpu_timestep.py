"""The force criterion of TimeStep on the GPU (src/timestep.cpp:18-38): dt = min(cflSound *
min_i h_i / v_sig_i, cflForce * min_i sqrt(h_i / |a_i|)) per run.

The device finds the force minimum with an FP32 pre-pass and evaluates the FP64 expression only
for the particles whose FP32 estimate lies within 2^-12 of the run's smallest estimate (and for
every particle outside the estimate's range).  These tests check that the result is the same FP64
number as the expression over all particles (numpy, IEEE FP64 operations in the device's order):
accelerations over 160 orders of magnitude, near-ties in the last bits of the quotient, zero,
signed-zero and NaN components, one run and batches of runs, in 1D, 2D and 3D."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DBL_MAX = np.finfo(np.float64).max


def _dt_force(acc, sml, cfl):
    """cflForce * sqrt(h / |a|) for |a| > 0, DBL_MAX otherwise; a^2 summed left to right."""
    a2 = np.zeros(acc.shape[0])
    for k in range(acc.shape[1]):
        a2 = a2 + acc[:, k] * acc[:, k]
    with np.errstate(all="ignore"):
        a = np.sqrt(a2)
        v = cfl * np.sqrt(sml / a)
    return np.where(a > 0.0, v, DBL_MAX)


def _expected_dt(acc, sml, counts, cfl_force, cfl_sound, hvs):
    out, b = [], 0
    v = _dt_force(acc, sml, cfl_force)
    for c in counts:
        seg = v[b:b + c]
        seg = seg[~np.isnan(seg)]
        df = seg.min() if seg.size else DBL_MAX
        ds = cfl_sound * hvs
        out.append(ds if ds < df else df)
        b += c
    return np.array(out)


def _case(dim):
    from sphcode_gb300 import ics
    if dim == 1:
        return ics.sod()
    if dim == 2:
        return ics.khi(32, 23)
    return ics.evrard(1500, seed=3)


def _accelerations(rng, n, dim, kind):
    if kind == "wide":
        # magnitudes 1e-80 .. 1e80 per component, random signs, some exact zeros
        acc = rng.choice([-1.0, 1.0], (n, dim)) * 10.0 ** rng.uniform(-80, 80, (n, dim))
        acc[rng.random((n, dim)) < 0.1] = 0.0
        sml = 10.0 ** rng.uniform(-3, 1, n)
    elif kind == "ties":
        # one quotient h/|a| repeated with perturbations in the last bits: every FP32 estimate is
        # the same number, the FP64 values differ
        base = rng.normal(size=dim)
        scale = 1.0 + rng.integers(0, 64, n) * 2.0 ** -52
        acc = base[None, :] * scale[:, None]
        sml = np.full(n, 0.0123456789) * (1.0 + rng.integers(0, 64, n) * 2.0 ** -52)
    else:
        # ordinary values with edge members: zero vectors, signed zeros, a NaN component, values
        # outside the FP32 estimate's range
        acc = rng.normal(size=(n, dim)) * 10.0 ** rng.uniform(-2, 2, (n, 1))
        sml = 10.0 ** rng.uniform(-2, -1, n)
        acc[0] = 0.0
        acc[1] = -0.0
        acc[2, 0] = np.nan
        acc[3] = 1e-200    # outside the FP32 estimate's range: always evaluated in FP64
        acc[4] = 1e-150
        sml[5] = 1e70
    return acc, sml


@pytest.mark.parametrize("kind", ["wide", "ties", "edges"])
@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("batch", [False, True])
def test_force_criterion_minimum_is_exact(gpu_lib, dim, kind, batch):
    from sphcode_gb300 import sphgpu
    p, f = _case(dim)
    n = int(np.asarray(f["mass"]).shape[0])
    rng = np.random.default_rng(dim * 100 + len(kind) + (7 if batch else 0))
    counts = [n] if not batch else [n // 3, n // 3, n - 2 * (n // 3)]
    acc, sml = _accelerations(rng, n, dim, kind)
    if batch:
        # a different scale in each run, so that each run has its own minimum
        b = 0
        for r, c in enumerate(counts):
            acc[b:b + c] *= 4.0 ** r
            b += c
    hvs = 1e300
    with sphgpu.GpuSimulation(p, f, precision="fp32", runs=counts if batch else None) as sim:
        sim.set("acc", acc)
        sim.set("sml", sml)
        for r in range(len(counts)):
            sim.set_scalar("h_per_v_sig", hvs, run=r)
        sim.timestep()
        got = np.array([sim.scalar("dt", run=r) for r in range(len(counts))])
    want = _expected_dt(acc, sml, counts, p.cfl_force, p.cfl_sound, hvs)
    assert np.array_equal(got, want), (got, want)


def test_force_criterion_twice_in_a_row(gpu_lib):
    """The per-run FP32 minimum is reset after each call: a second call on larger accelerations
    (a smaller dt) and a third on smaller ones (a larger dt) give their own minima."""
    from sphcode_gb300 import sphgpu
    p, f = _case(2)
    n = int(np.asarray(f["mass"]).shape[0])
    rng = np.random.default_rng(11)
    acc = rng.normal(size=(n, 2))
    sml = 10.0 ** rng.uniform(-2, -1, n)
    with sphgpu.GpuSimulation(p, f, precision="fp64") as sim:
        sim.set("sml", sml)
        for scale in (1.0, 100.0, 0.01):
            sim.set("acc", acc * scale)
            sim.set_scalar("h_per_v_sig", 1e300)
            sim.timestep()
            want = _expected_dt(acc * scale, sml, [n], p.cfl_force, p.cfl_sound, 1e300)[0]
            assert sim.scalar("dt") == want
