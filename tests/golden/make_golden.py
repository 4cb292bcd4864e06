"""Generate the golden fixtures of tests/golden/ from the reference's own modules.

The reference (mitchiinaga/sphcode) ships no golden vectors or known-answer tests for its hot
path; its only test prints kernel finite-difference errors (test/kernel_test/kernel_test.cpp).
These fixtures are therefore produced by running the reference's unmodified translation units
(src/bhtree.cpp, src/pre_interaction.cpp, src/fluid_force.cpp, src/gravity_force.cpp,
src/timestep.cpp, src/disph/*, src/gsph/*), compiled by oracle/build_ref.sh with strict IEEE
FP64 flags and driven through oracle/ref_harness.cpp, on small seeded inputs of the benchmark
workloads.  Each fixture stores the per-particle fields after Solver::initialize and after two
Solver::integrate steps, the smoothing-length guess inputs, and the exhaustive neighbour sets.

    python tests/golden/make_golden.py        (needs oracle/_ref built from the reference)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from sphcode_gb300 import ics  # noqa: E402

CASES = {
    "sod_ssph_1d": lambda: ics.sod(200, 25),
    "khi_disph_ac_2d": lambda: ics.khi(32, 23),
    "gresho_ssph_2d": lambda: ics.gresho(24),
    "evrard_disph_grav_3d": lambda: ics.evrard(1500, seed=11),
    "gsph_tube_1d": lambda: ics.shock_tube_gsph(150, 40, 1.0, 0.3, 1.0, 0.2),
}


def fields_of(p):
    names = ["pos", "vel", "ene", "dens", "sml", "pres", "acc", "dene", "sound", "neighbor"]
    if p.sph_type != "gsph":
        names += ["gradh", "alpha", "balsara"]
    else:
        names += ["grad_d", "grad_p", "grad_v"]
    if p.use_gravity:
        names += ["phi"]
    return names


def main():
    if not pyoracle.reference_available():
        pyoracle.build_reference()
    for name, make in CASES.items():
        p, f = make()
        sim = pyoracle.OracleSim(p, f, kind="ref")
        sim.initialize()
        out = {}
        for fld in fields_of(p):
            out[f"init/{fld}"] = sim.get(fld)
        out["init/h_per_v_sig"] = np.array(sim.scalar("h_per_v_sig"))
        c, l = sim.neighbors(0, exhaustive=True, cap=256)
        out["init/nb_count"] = c
        out["init/nb_list"] = np.concatenate([np.sort(l[i, :c[i]]) for i in range(sim.n)]).astype(np.int32)
        for _ in range(2):
            sim.step()
        for fld in fields_of(p):
            out[f"step2/{fld}"] = sim.get(fld)
        out["step2/time"] = np.array(sim.scalar("time"))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, sim.n, "particles")


if __name__ == "__main__":
    main()
