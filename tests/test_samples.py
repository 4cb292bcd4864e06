"""The reference's six samples: their JSON parameter files read by the Boost-free reader, and the
host restatement of their initial conditions (src/sample/*.cpp).

Parameters: each file is read as `sph <sample>` reads it (Solver::read_parameterfile,
src/solver.cpp:155-299); the expected values below are the file's keys with the reader's defaults
for the missing ones (outputTime = (endTime - startTime) / 100, energyTime = outputTime,
cflSound 0.3, cflForce 0.125, useBalsaraSwitch true, useTimeDependentAV false,
useArtificialConductivity false, maxTreeLevel 20, leafParticleNumber 1, iterativeSmoothingLength
true, useGravity false; G 1 and theta 0.5 when gravity is on; alphaMax 2, alphaMin 0.1,
epsilonAV 0.2 when the time-dependent AV is on) and the sample's particle count N.

Initial conditions: particle counts, masses and states of each generator as the reference's
loops produce them, and the pairing-instability offsets against the draws of the GNU C++
library's std::mt19937 / std::uniform_real_distribution (tests/golden/samples/mt19937_uniform.npz).
"""
import math
import os

import numpy as np
import pytest

from conftest import reference_root
from sphcode_gb300 import ics
from sphcode_gb300.params import SPHParameters

G53 = 1.66666666666666666666666666666666667

EXPECTED = {
    "shock_tube": dict(dim=1, end_time=0.2, output_time=0.002, sph_type="ssph", av_alpha=1.0,
                       neighbor_number=4, gamma=1.4, kernel="cubic_spline", periodic=True,
                       iterative_sml=True, use_tdav=False, use_balsara=True, leaf_num=1,
                       range_min=[-0.5], range_max=[1.5], use_gravity=False, sample_n=50),
    "gresho_chan_vortex": dict(dim=2, end_time=1.0, output_time=0.01, sph_type="ssph",
                               neighbor_number=32, use_balsara=True, leaf_num=32, gamma=G53,
                               kernel="wendland", periodic=True, range_min=[-0.5, -0.5],
                               range_max=[0.5, 0.5], use_tdav=False, sample_n=64),
    "pairing_instability": dict(dim=2, end_time=1.0, sph_type="ssph", neighbor_number=32,
                                leaf_num=32, gamma=G53, kernel="cubic_spline", periodic=True,
                                range_min=[-0.5, -0.5], range_max=[0.5, 0.5], use_balsara=True,
                                sample_n=64),
    "hydrostatic": dict(dim=2, end_time=8.0, output_time=0.08, sph_type="disph", neighbor_number=32,
                        use_balsara=True, leaf_num=16, gamma=G53, kernel="wendland", periodic=True,
                        range_min=[-0.5, -0.5], range_max=[0.5, 0.5], sample_n=32),
    "khi": dict(dim=2, end_time=3.0, output_time=0.1, energy_time=0.1, sph_type="ssph",
                neighbor_number=32, use_balsara=True, use_tdav=True, alpha_max=2.0, alpha_min=0.1,
                epsilon_av=0.2, use_ac=False, leaf_num=16, gamma=G53, kernel="wendland",
                periodic=True, range_min=[0.0, 0.0], range_max=[1.0, 1.0], sample_n=256),
    "evrard": dict(dim=3, end_time=3.0, sph_type="disph", neighbor_number=32, use_balsara=True,
                   use_tdav=True, alpha_max=2.0, alpha_min=0.1, epsilon_av=0.2, use_ac=False,
                   leaf_num=32, gamma=G53, kernel="wendland", periodic=False, use_gravity=True,
                   g_constant=1.0, theta=0.5, sample_n=30),
}


@pytest.fixture(scope="module")
def root():
    r = reference_root()
    if r is None:
        pytest.skip("no reference sample/ directory (SPHCODE_REFERENCE or the oracle snapshot)")
    return r


@pytest.mark.parametrize("name", list(EXPECTED))
def test_sample_parameter_files(root, name):
    p = SPHParameters.from_json(name, ics.SAMPLE_DIM[name], sample_root=root)
    want = EXPECTED[name]
    D = want["dim"]
    assert p.sample == name
    assert p.output_directory == f"sample/{name}/results"
    assert p.start_time == 0.0 and p.cfl_sound == 0.3 and p.cfl_force == 0.125 and p.av_alpha == 1.0
    assert p.max_level == 20
    if "energy_time" not in want:
        assert p.energy_time == p.output_time
    for k, v in want.items():
        got = getattr(p, k)
        if k in ("range_min", "range_max"):
            assert got[:D] == v, (name, k, got)
        elif isinstance(v, float):
            assert got == pytest.approx(v, rel=1e-15), (name, k, got)
        else:
            assert got == v, (name, k, got)


def test_sample_counts_and_states(root):
    p, f = ics.reference_sample("shock_tube", root)
    N = 50
    assert f["mass"].size == 10 * N
    left = f["dens"] == 1.0
    assert int(left.sum()) == 8 * N and np.all(f["dens"][~left] == 0.25)
    assert np.all(f["pres"][~left] == 0.1795) and np.all(np.diff(f["pos"][:, 0]) > 0)
    assert f["pos"][0, 0] == -0.5 + 0.5 / N * 0.25 * 0.5
    # the left lattice ends where x first passes 0.5; the right one starts half a spacing after
    assert f["pos"][8 * N, 0] == 0.5 + 0.5 / N * 0.5

    p, f = ics.reference_sample("khi", root)
    N = 256
    assert f["mass"].size == N * N * 3 // 4
    inner = f["dens"] == 2.0
    assert np.all(f["vel"][inner, 0] == 0.5) and np.all(f["vel"][~inner, 0] == -0.5)
    assert np.all((f["pos"][inner, 1] > 0.25) & (f["pos"][inner, 1] < 0.75))
    assert int(inner.sum()) == N * N // 2
    assert f["mass"][0] == 1.5 / (N * N * 3 // 4) and np.all(f["pres"] == 2.5)

    p, f = ics.reference_sample("evrard", root)
    r = np.sqrt((f["pos"] ** 2).sum(1))
    assert np.all(r <= 1.0) and f["mass"].sum() == pytest.approx(1.0, rel=1e-12)
    assert np.all(f["ene"] == 0.05) and np.allclose(f["dens"], 1.0 / (2 * np.pi * r))
    # the stretched lattice: the cells of the 30^3 lattice inside the unit sphere
    c = (np.arange(30) + 0.5) * (2.0 / 30) - 1.0
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    assert f["mass"].size == int(np.sum(np.sqrt(X * X + Y * Y + Z * Z) <= 1.0))

    p, f = ics.reference_sample("gresho_chan_vortex", root)
    r = np.sqrt((f["pos"] ** 2).sum(1))
    vphi = np.where(r < 0.2, 5 * r, np.where(r < 0.4, 2 - 5 * r, 0.0))
    assert np.allclose(np.sqrt((f["vel"] ** 2).sum(1)), vphi, rtol=1e-14, atol=1e-15)
    assert f["mass"].size == 64 * 64

    p, f = ics.reference_sample("hydrostatic", root)
    dense = f["dens"] == 4.0
    assert int(dense.sum()) == 32 * 32 and f["mass"][0] == 1.0 / (32 * 32)
    inside = (np.abs(f["pos"][:, 0]) < 0.25) & (np.abs(f["pos"][:, 1]) < 0.25)
    assert np.array_equal(dense, inside)
    assert int((~dense).sum()) == 32 * 32 - 16 * 16   # the ambient lattice skips the square

    p, f = ics.reference_sample("pairing_instability", root)
    assert f["mass"].size == 64 * 64 and np.all(f["dens"] == 1.0)


def test_mt19937_and_uniform_draws_match_the_cxx_library():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "samples", "mt19937_uniform.npz"))
    eng = ics._MT19937(1)
    assert [eng() for _ in range(16)] == [int(x) for x in g["raw"]]
    eng = ics._MT19937(1)
    dx = 1.0 / 64
    draws = [ics._uniform_real(eng, -dx * 0.05, dx * 0.05) for _ in range(g["draws"].size)]
    assert np.array_equal(np.array(draws), g["draws"])
    # the C++ standard's check value: the 10000th output of a default-seeded mt19937
    eng = ics._MT19937(5489)
    for _ in range(9999):
        eng()
    assert eng() == 4123659995


def test_pairing_offsets_are_the_library_draws(root):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "samples", "mt19937_uniform.npz"))["draws"]
    p, f = ics.reference_sample("pairing_instability", root)
    N, dx = 64, 1.0 / 64
    x, y, i = -0.5 + dx * 0.5, -0.5 + dx * 0.5, 0
    for k in range(N * N):
        assert f["pos"][k, 0] == x + g[2 * k] and f["pos"][k, 1] == y + g[2 * k + 1]
        x += dx
        if x > 0.5:
            x = -0.5 + dx * 0.5
            y += dx
