"""The reference's host-side interface over the GPU library: Simulation, Module and its stages,
Solver, Output.

Mirrors sph::Module (include/module.hpp:10-14: ``initialize(param)``, ``calculation(sim)``),
sph::Simulation (include/simulation.hpp:17-45), the Module subclasses selected by SPHType in
Solver::initialize (src/solver.cpp:359-370), Solver::run / integrate / predict / correct
(src/solver.cpp:301-474) and Output (src/output.cpp:14-90).  Every calculation runs on the
device through the C-ABI (sphgpu.py); the particle state stays resident between calls and is
read back only where a caller asks for it (get_particles, output).
"""
from __future__ import annotations

import os
from typing import Dict, Optional, Sequence

import numpy as np

from .params import SPHParameters
from .sphgpu import GpuSimulation


class Simulation:
    """Device-resident counterpart of sph::Simulation: particles, time, dt, h/v_sig."""

    def __init__(self, param: SPHParameters, fields: Dict[str, np.ndarray], precision: str = "fp32",
                 runs: Optional[Sequence[int]] = None):
        self.param = param
        self.gpu = GpuSimulation(param, fields, precision=precision, runs=runs)

    # Simulation::get_particles (a host copy of the fields the reference's particles carry)
    def get_particles(self, names=("pos", "vel", "acc", "mass", "dens", "pres", "ene", "sml", "neighbor",
                                   "alpha", "gradh", "phi", "balsara", "sound", "dene")) -> Dict[str, np.ndarray]:
        return {k: self.gpu.get(k) for k in names}

    def get_particle_num(self) -> int:
        return self.gpu.n

    def get_time(self, run: int = 0) -> float:
        return self.gpu.scalar("time", run)

    def get_dt(self, run: int = 0) -> float:
        return self.gpu.scalar("dt", run)

    def set_dt(self, dt: float, run: int = 0) -> None:
        self.gpu.set_scalar("dt", dt, run)

    def get_h_per_v_sig(self, run: int = 0) -> float:
        return self.gpu.scalar("h_per_v_sig", run)

    def set_h_per_v_sig(self, v: float, run: int = 0) -> None:
        self.gpu.set_scalar("h_per_v_sig", v, run)

    def update_time(self, run: int = 0) -> None:
        """Simulation::update_time (src/simulation.cpp:32-35)."""
        self.gpu.set_scalar("time", self.get_time(run) + self.get_dt(run), run)

    def make_tree(self) -> None:
        """Simulation::make_tree (src/simulation.cpp:37-40)."""
        self.gpu.make_tree()

    def close(self) -> None:
        self.gpu.close()


class Module:
    """sph::Module."""

    def initialize(self, param: SPHParameters) -> None:
        self.param = param

    def calculation(self, sim: Simulation) -> None:
        raise NotImplementedError


class PreInteraction(Module):
    """PreInteraction of the parameter's SPH type (ssph src/pre_interaction.cpp, disph
    src/disph/d_pre_interaction.cpp, gsph src/gsph/g_pre_interaction.cpp), including the first-call
    initial smoothing and the closing BHTree::set_kernel."""

    def calculation(self, sim: Simulation) -> None:
        sim.gpu.pre_interaction()


class FluidForce(Module):
    """FluidForce of the parameter's SPH type (src/fluid_force.cpp, src/disph/d_fluid_force.cpp,
    src/gsph/g_fluid_force.cpp)."""

    def calculation(self, sim: Simulation) -> None:
        sim.gpu.fluid_force()


class GravityForce(Module):
    """GravityForce (src/gravity_force.cpp:52-89); returns at once without useGravity."""

    def calculation(self, sim: Simulation) -> None:
        sim.gpu.gravity_force()


class TimeStep(Module):
    """TimeStep (src/timestep.cpp:18-38)."""

    def calculation(self, sim: Simulation) -> None:
        sim.gpu.timestep()


class Output:
    """Particle dumps ``%05d.dat`` and ``energy.dat`` in the reference's text formats
    (src/output.cpp:14-90)."""

    def __init__(self, directory: str, count: int = 0):
        self.dir = directory
        self.count = count
        os.makedirs(directory, exist_ok=True)
        self._energy = open(os.path.join(directory, "energy.dat"), "w")
        self._energy.write("# time kinetic thermal potential total\n")

    def output_particle(self, sim: Simulation) -> str:
        """Columns: pos, vel, acc (DIM each), mass, dens, pres, ene, sml, id, neighbor, alpha,
        gradh, in particle (id) order, after a ``# time`` line (src/output.cpp:14-32,46-64)."""
        p = sim.get_particles(("pos", "vel", "acc", "mass", "dens", "pres", "ene", "sml", "neighbor",
                               "alpha", "gradh"))
        n = sim.get_particle_num()
        cols = [p["pos"], p["vel"], p["acc"]]
        cols += [p[k].reshape(n, 1) for k in ("mass", "dens", "pres", "ene", "sml")]
        cols += [np.arange(n, dtype=np.float64).reshape(n, 1), p["neighbor"].reshape(n, 1)]
        cols += [p[k].reshape(n, 1) for k in ("alpha", "gradh")]
        table = np.hstack(cols)
        path = os.path.join(self.dir, "%05d.dat" % self.count)
        dim = p["pos"].shape[1]
        int_cols = {3 * dim + 5, 3 * dim + 6}
        with open(path, "w") as f:
            f.write("# %r\n" % float(sim.get_time()))
            for row in table:
                f.write(" ".join(("%d" % int(v)) if c in int_cols else repr(float(v))
                                 for c, v in enumerate(row)) + " \n")
        self.count += 1
        return path

    def output_energy(self, sim: Simulation) -> np.ndarray:
        """``time kinetic thermal potential total`` (src/output.cpp:66-90)."""
        e = sim.gpu.energy()
        self._energy.write(" ".join(repr(float(x)) for x in (sim.get_time(), e[0], e[1], e[2], e[3])) + "\n")
        self._energy.flush()
        return e

    def close(self) -> None:
        self._energy.close()


class Solver:
    """Solver::run / initialize / integrate (src/solver.cpp:301-474) over device-resident state.

    ``integrate`` calls the modules one by one like the reference; ``run`` advances whole steps on
    the device (one CUDA graph per step) and reads back only for output."""

    def __init__(self, param: SPHParameters, fields: Dict[str, np.ndarray], precision: str = "fp32",
                 output_dir: Optional[str] = None):
        self.param = param
        self.sim = Simulation(param, fields, precision)
        self.timestep, self.pre, self.fforce, self.gforce = TimeStep(), PreInteraction(), FluidForce(), GravityForce()
        for m in (self.timestep, self.pre, self.fforce, self.gforce):
            m.initialize(param)
        self.output = Output(output_dir) if output_dir else None

    def initialize(self) -> None:
        """Field start-up, tree, first Pre / Fluid / Gravity (src/solver.cpp:392-414)."""
        self.sim.gpu.initialize()

    def integrate(self) -> None:
        """One Solver::integrate (src/solver.cpp:417-429) through the modules."""
        self.timestep.calculation(self.sim)
        self.sim.gpu.predict()
        self.sim.make_tree()
        self.pre.calculation(self.sim)
        self.fforce.calculation(self.sim)
        self.gforce.calculation(self.sim)
        self.sim.gpu.correct()
        self.sim.update_time()

    def run(self, max_steps: Optional[int] = None) -> int:
        """Time loop to endTime with output at outputTime / energyTime (src/solver.cpp:301-351).
        Returns the number of steps taken."""
        self.initialize()
        t_end = self.param.end_time
        t_out = self.param.output_time
        t_ene = self.param.energy_time
        if self.output:
            self.output.output_particle(self.sim)
            self.output.output_energy(self.sim)
        loop = 0
        t = self.sim.get_time()
        while t < t_end and (max_steps is None or loop < max_steps):
            self.sim.gpu.step(1)
            loop += 1
            t = self.sim.get_time()
            if self.output and t > t_out:
                self.output.output_particle(self.sim)
                t_out += self.param.output_time
            if self.output and t > t_ene:
                self.output.output_energy(self.sim)
                t_ene += self.param.energy_time
        return loop

    def close(self) -> None:
        if self.output:
            self.output.close()
        self.sim.close()
