"""The Boost-free reader of the reference's JSON parameter files (keys, defaults, conditional
reads and errors of Solver::read_parameterfile, src/solver.cpp:155-299)."""
import json

import pytest

from sphcode_gb300.params import ParameterError, SPHParameters


def _write(tmp_path, d):
    p = tmp_path / "p.json"
    p.write_text(json.dumps(d))
    return str(p)


def test_defaults_and_required(tmp_path):
    p = SPHParameters.from_json(_write(tmp_path, {"outputDirectory": "o", "endTime": 1.0, "gamma": 1.4}), dim=2)
    assert p.sph_type == "ssph" and p.kernel == "cubic_spline"
    assert p.cfl_sound == 0.3 and p.cfl_force == 0.125 and p.av_alpha == 1.0
    assert p.use_balsara and not p.use_tdav and not p.use_ac and not p.use_gravity
    assert p.max_level == 20 and p.leaf_num == 1 and p.neighbor_number == 32
    assert p.iterative_sml and not p.periodic
    assert p.output_time == pytest.approx(0.01) and p.energy_time == p.output_time
    with pytest.raises(ParameterError):
        SPHParameters.from_json(_write(tmp_path, {"outputDirectory": "o", "gamma": 1.4}), dim=2)


def test_conditional_reads(tmp_path):
    base = {"outputDirectory": "o", "endTime": 1.0, "gamma": 5 / 3}
    # alphaMax/alphaMin/epsilonAV only with useTimeDependentAV
    p = SPHParameters.from_json(_write(tmp_path, dict(base, alphaMax=3.0)), dim=3)
    assert p.alpha_max == 2.0
    p = SPHParameters.from_json(_write(tmp_path, dict(base, useTimeDependentAV=True, alphaMax=3.0,
                                                      alphaMin=0.2, epsilonAV=0.1)), dim=3)
    assert (p.alpha_max, p.alpha_min, p.epsilon_av) == (3.0, 0.2, 0.1)
    with pytest.raises(ParameterError):
        SPHParameters.from_json(_write(tmp_path, dict(base, useTimeDependentAV=True, alphaMax=0.05)), dim=3)
    # G/theta only with useGravity
    p = SPHParameters.from_json(_write(tmp_path, dict(base, useGravity=True, G=2.0, theta=0.7)), dim=3)
    assert (p.g_constant, p.theta) == (2.0, 0.7)
    # periodic ranges must have DIM entries
    p = SPHParameters.from_json(_write(tmp_path, dict(base, periodic=True, rangeMin=[-0.5, -0.5],
                                                      rangeMax=[0.5, 0.5])), dim=2)
    assert p.range_min[:2] == [-0.5, -0.5] and p.range_max[:2] == [0.5, 0.5]
    with pytest.raises(ParameterError):
        SPHParameters.from_json(_write(tmp_path, dict(base, periodic=True, rangeMin=[0], rangeMax=[1])), dim=2)
    with pytest.raises(ParameterError):
        SPHParameters.from_json(_write(tmp_path, dict(base, SPHType="bogus")), dim=2)
    p = SPHParameters.from_json(_write(tmp_path, dict(base, SPHType="gsph", use2ndOrderGSPH=False)), dim=1)
    assert p.sph_type == "gsph" and not p.gsph_2nd_order


def test_c_struct_round_trip():
    from sphcode_gb300.params import CParams
    p = SPHParameters(dim=3, sph_type="disph", kernel="wendland", gamma=5 / 3, neighbor_number=50,
                      use_gravity=True, theta=0.5, leaf_num=32)
    c = p.to_c(CParams)
    assert (c.sph_type, c.kernel, c.neighbor_number, c.use_gravity, c.leaf_num) == (1, 1, 50, 1, 32)
    assert c.gamma == pytest.approx(5 / 3) and c.theta == 0.5
