"""SPHParameters and the JSON parameter-file reader.

Mirrors ``sph::SPHParameters`` (include/parameters.hpp:20-79) and ``Solver::read_parameterfile``
(src/solver.cpp:155-299): the same JSON keys, the same defaults, the same validation errors, and
the same conditional reads (``alphaMax``/``alphaMin``/``epsilonAV`` only when
``useTimeDependentAV``; ``alphaAC`` only with ``useArtificialConductivity``; ``G``/``theta`` only
with ``useGravity``; ``use2ndOrderGSPH`` only for ``gsph``).  The reference reads the files with
Boost.PropertyTree; this reader uses the standard ``json`` module, so the parameter files of the
reference's ``sample/`` directory load unchanged.
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Union

SPH_TYPES = {"ssph": 0, "disph": 1, "gsph": 2}
KERNELS = {"cubic_spline": 0, "wendland": 1}

# Sample names accepted in place of a path, with the default particle count the reference
# applies when the file has no "N" (src/solver.cpp:164-187).
SAMPLES = {
    "shock_tube": 100,
    "gresho_chan_vortex": 64,
    "pairing_instability": 64,
    "hydrostatic": 32,
    "khi": 128,
    "evrard": 20,
}


class ParameterError(ValueError):
    """Raised where the reference raises THROW_ERROR while reading parameters."""


@dataclass
class SPHParameters:
    dim: int = 3
    output_directory: str = ""
    start_time: float = 0.0
    end_time: float = 0.0
    output_time: float = 0.0
    energy_time: float = 0.0
    sph_type: str = "ssph"
    cfl_sound: float = 0.3
    cfl_force: float = 0.125
    av_alpha: float = 1.0
    use_balsara: bool = True
    use_tdav: bool = False
    alpha_max: float = 2.0
    alpha_min: float = 0.1
    epsilon_av: float = 0.2
    use_ac: bool = False
    alpha_ac: float = 1.0
    max_level: int = 20
    leaf_num: int = 1
    neighbor_number: int = 32
    gamma: float = 1.4
    kernel: str = "cubic_spline"
    iterative_sml: bool = True
    periodic: bool = False
    range_min: List[float] = field(default_factory=lambda: [0.0, 0.0, 0.0])
    range_max: List[float] = field(default_factory=lambda: [0.0, 0.0, 0.0])
    use_gravity: bool = False
    g_constant: float = 1.0
    theta: float = 0.5
    gsph_2nd_order: bool = True
    # sample bookkeeping (Solver::m_sample, m_sample_parameters["N"])
    sample: Optional[str] = None
    sample_n: Optional[int] = None

    @property
    def sph_type_id(self) -> int:
        return SPH_TYPES[self.sph_type]

    @property
    def kernel_id(self) -> int:
        return KERNELS[self.kernel]

    # ------------------------------------------------------------------------------------------
    @classmethod
    def from_dict(cls, d: Dict[str, Any], dim: int) -> "SPHParameters":
        """Apply ``Solver::read_parameterfile``'s reads to an already-parsed JSON object."""
        p = cls(dim=dim)

        def get(key, default=None, required=False):
            if key in d:
                return d[key]
            if required:
                raise ParameterError(f"No such node ({key})")
            return default

        p.output_directory = str(get("outputDirectory", required=True))
        p.start_time = float(get("startTime", 0.0))
        p.end_time = float(get("endTime", required=True))
        if p.end_time < p.start_time:
            raise ParameterError("endTime < startTime")
        p.output_time = float(get("outputTime", (p.end_time - p.start_time) / 100))
        p.energy_time = float(get("energyTime", p.output_time))
        p.sph_type = str(get("SPHType", "ssph"))
        if p.sph_type not in SPH_TYPES:
            raise ParameterError("Unknown SPH type")
        p.cfl_sound = float(get("cflSound", 0.3))
        p.cfl_force = float(get("cflForce", 0.125))
        p.av_alpha = float(get("avAlpha", 1.0))
        p.use_balsara = bool(get("useBalsaraSwitch", True))
        p.use_tdav = bool(get("useTimeDependentAV", False))
        if p.use_tdav:
            p.alpha_max = float(get("alphaMax", 2.0))
            p.alpha_min = float(get("alphaMin", 0.1))
            if p.alpha_max < p.alpha_min:
                raise ParameterError("alphaMax < alphaMin")
            p.epsilon_av = float(get("epsilonAV", 0.2))
        p.use_ac = bool(get("useArtificialConductivity", False))
        if p.use_ac:
            p.alpha_ac = float(get("alphaAC", 1.0))
        p.max_level = int(get("maxTreeLevel", 20))
        p.leaf_num = int(get("leafParticleNumber", 1))
        p.neighbor_number = int(get("neighborNumber", 32))
        p.gamma = float(get("gamma", required=True))
        p.kernel = str(get("kernel", "cubic_spline"))
        if p.kernel not in KERNELS:
            raise ParameterError("kernel is unknown.")
        p.iterative_sml = bool(get("iterativeSmoothingLength", True))
        p.periodic = bool(get("periodic", False))
        if p.periodic:
            rmax = list(get("rangeMax", required=True))
            if len(rmax) != dim:
                raise ParameterError("rangeMax != DIM")
            rmin = list(get("rangeMin", required=True))
            if len(rmin) != dim:
                raise ParameterError("rangeMax != DIM")   # the reference's message (solver.cpp:278)
            p.range_max = [float(x) for x in rmax] + [0.0] * (3 - dim)
            p.range_min = [float(x) for x in rmin] + [0.0] * (3 - dim)
        p.use_gravity = bool(get("useGravity", False))
        if p.use_gravity:
            p.g_constant = float(get("G", 1.0))
            p.theta = float(get("theta", 0.5))
        if p.sph_type == "gsph":
            p.gsph_2nd_order = bool(get("use2ndOrderGSPH", True))
        return p

    @classmethod
    def from_json(cls, path_or_sample: Union[str, os.PathLike], dim: int,
                  sample_root: Optional[str] = None) -> "SPHParameters":
        """Read a parameter file, or a sample name resolved to ``sample/<name>/<name>.json``
        under ``sample_root`` (src/solver.cpp:163-191)."""
        name = os.fspath(path_or_sample)
        sample = None
        if name in SAMPLES:
            sample = name
            root = sample_root or "."
            name = os.path.join(root, "sample", sample, sample + ".json")
        with open(name, "r") as f:
            d = json.load(f)
        p = cls.from_dict(d, dim)
        if sample is not None:
            p.sample = sample
            p.sample_n = int(d.get("N", SAMPLES[sample]))
        return p

    # ------------------------------------------------------------------------------------------
    def to_c(self, struct_type):
        """Fill a ctypes structure with the C layout shared by the library and the oracle."""
        s = struct_type()
        s.sph_type = self.sph_type_id
        s.kernel = self.kernel_id
        s.cfl_sound = self.cfl_sound
        s.cfl_force = self.cfl_force
        s.av_alpha = self.av_alpha
        s.use_balsara = int(self.use_balsara)
        s.use_tdav = int(self.use_tdav)
        s.alpha_max = self.alpha_max
        s.alpha_min = self.alpha_min
        s.epsilon_av = self.epsilon_av
        s.use_ac = int(self.use_ac)
        s.alpha_ac = self.alpha_ac
        s.max_level = self.max_level
        s.leaf_num = self.leaf_num
        s.neighbor_number = self.neighbor_number
        s.gamma = self.gamma
        s.iterative_sml = int(self.iterative_sml)
        s.periodic = int(self.periodic)
        for k in range(3):
            s.range_min[k] = float(self.range_min[k]) if k < len(self.range_min) else 0.0
            s.range_max[k] = float(self.range_max[k]) if k < len(self.range_max) else 0.0
        s.use_gravity = int(self.use_gravity)
        s.g_constant = self.g_constant
        s.theta = self.theta
        s.gsph_2nd_order = int(self.gsph_2nd_order)
        return s


class CParams(ctypes.Structure):
    """C layout of ``sphgpu_params`` (include/sphgpu.h) — identical to the oracle's struct."""
    _fields_ = [
        ("sph_type", ctypes.c_int), ("kernel", ctypes.c_int),
        ("cfl_sound", ctypes.c_double), ("cfl_force", ctypes.c_double),
        ("av_alpha", ctypes.c_double), ("use_balsara", ctypes.c_int), ("use_tdav", ctypes.c_int),
        ("alpha_max", ctypes.c_double), ("alpha_min", ctypes.c_double),
        ("epsilon_av", ctypes.c_double), ("use_ac", ctypes.c_int), ("alpha_ac", ctypes.c_double),
        ("max_level", ctypes.c_int), ("leaf_num", ctypes.c_int),
        ("neighbor_number", ctypes.c_int), ("gamma", ctypes.c_double),
        ("iterative_sml", ctypes.c_int), ("periodic", ctypes.c_int),
        ("range_min", ctypes.c_double * 3), ("range_max", ctypes.c_double * 3),
        ("use_gravity", ctypes.c_int), ("g_constant", ctypes.c_double),
        ("theta", ctypes.c_double), ("gsph_2nd_order", ctypes.c_int),
    ]
