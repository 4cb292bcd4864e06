"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Loads either the C port (oracle/sph_oracle.c, built here into oracle/_build/) or the reference's
own modules (oracle/_ref/, built by oracle/build_ref.sh where the reference sources exist) behind
one Python class, so tests can drive both through identical calls.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")

FIELDS = ["pos", "vel", "vel_p", "acc", "mass", "dens", "pres", "ene", "ene_p", "dene", "sml",
          "sound", "balsara", "alpha", "gradh", "phi", "neighbor", "grad_d", "grad_p", "grad_v"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
VECTOR = {"pos", "vel", "vel_p", "acc", "grad_d", "grad_p"}
STAGES = {"timestep": 0, "predict": 1, "make_tree": 2, "pre": 3, "fluid": 4, "gravity": 5,
          "correct": 6, "init_fields": 7}

_lock = threading.Lock()
_libs: Dict[str, ctypes.CDLL] = {}


class OrcParams(ctypes.Structure):
    """orc_params of oracle/sph_oracle.h."""
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


PORT_FLAGS = {
    # parity flavour: IEEE FP64 without contraction, like the strict reference build
    "strict": ["-O2", "-fno-fast-math", "-ffp-contract=off"],
    # timing flavour: the reference Makefile's optimisation flags (Makefile:4-10)
    "fast": ["-O3", "-funroll-loops", "-ffast-math"],
}


def port_path(flavor: str = "strict") -> str:
    return os.path.join(BUILD, f"liborc_{flavor}.so")


def build_port(force: bool = False) -> None:
    """Compile oracle/sph_oracle.c for DIM = 1, 2, 3 into one shared library per flavour."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "sph_oracle.c")
    hdr = os.path.join(HERE, "sph_oracle.h")
    procs = []
    for flavor, flags in PORT_FLAGS.items():
        out = port_path(flavor)
        if (not force and os.path.exists(out)
                and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
            continue
        objs = []
        for d in (1, 2, 3):
            obj = os.path.join(BUILD, f"orc_{flavor}_d{d}.o")
            objs.append(obj)
            procs.append((out, objs, subprocess.Popen(
                ["gcc", "-std=c99", "-fPIC", "-fopenmp", *flags, f"-DDIM={d}", "-I", HERE,
                 "-c", src, "-o", obj])))
    for _, _, p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle port build failed")
    done = set()
    for out, objs, _ in procs:
        if out in done:
            continue
        done.add(out)
        subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", out + ".tmp", *objs])
        os.replace(out + ".tmp", out)


def build_reference(src: Optional[str] = None) -> bool:
    """Run the oracle/_ref recipe on the reference checkout `src` (else $SPHCODE_REFERENCE, else
    the snapshot an earlier build kept in oracle/_ref/snapshot).  Returns availability."""
    script = os.path.join(HERE, "build_ref.sh")
    src = src or os.environ.get("SPHCODE_REFERENCE", "")
    if not (src and os.path.exists(os.path.join(src, "include", "defines.hpp"))):
        snap = os.path.join(REF, "snapshot")
        if os.path.exists(os.path.join(snap, "include", "defines.hpp")):
            src = snap
        else:
            return reference_available()
    if _reference_up_to_date(src):
        return reference_available()
    env = dict(os.environ, SPHCODE_REFERENCE=src)
    subprocess.check_call(["bash", script], env=env, stdout=subprocess.DEVNULL)
    return reference_available()


def _reference_up_to_date(src: str) -> bool:
    """True when every library of the recipe is newer than its inputs (the recipe, the harness,
    the reference sources and headers, and for the GPU-module flavour the sphgpu library)."""
    root = os.path.dirname(HERE)
    gpu_lib = os.path.join(root, "sphcode_gb300", "_lib", "libsphgpu.so")
    outs = [os.path.join(REF, f"libref_{fl}_d{d}.so") for fl in ("strict", "fast") for d in (1, 2, 3)]
    ins = [os.path.join(HERE, "build_ref.sh"), os.path.join(HERE, "ref_harness.cpp"),
           os.path.join(HERE, "sph_oracle.h")]
    for sub in ("src", "include"):
        for dp, _, fns in os.walk(os.path.join(src, sub)):
            ins += [os.path.join(dp, fn) for fn in fns]
    if os.path.exists(gpu_lib):
        outs += [os.path.join(REF, f"libref_gpu_d{d}.so") for d in (1, 2, 3)]
        cxx = os.path.join(root, "sphcode_gb300", "cxx")
        ins += [gpu_lib, os.path.join(root, "include", "sphgpu.h")]
        ins += [os.path.join(cxx, fn) for fn in os.listdir(cxx)]
    if not all(os.path.exists(o) for o in outs):
        return False
    return min(os.path.getmtime(o) for o in outs) > max(os.path.getmtime(i) for i in ins)


def gpu_modules_available() -> bool:
    """The reference Solver glue with the GPU Module drop-ins (libref_gpu_dD.so) is built."""
    return all(os.path.exists(os.path.join(REF, f"libref_gpu_d{d}.so")) for d in (1, 2, 3))


def reference_available(flavor: str = "strict") -> bool:
    return all(os.path.exists(os.path.join(REF, f"libref_{flavor}_d{d}.so")) for d in (1, 2, 3))


def _load(kind: str, flavor: str) -> ctypes.CDLL:
    key = f"{kind}:{flavor}"
    with _lock:
        if key in _libs:
            return _libs[key]
        if kind == "port":
            if not os.path.exists(port_path(flavor)):
                build_port()
            lib = ctypes.CDLL(port_path(flavor))
            _libs[key] = lib
        else:
            libs = []
            for d in (1, 2, 3):
                path = os.path.join(REF, f"libref_{'gpu' if kind == 'gpumod' else flavor}_d{d}.so")
                if not os.path.exists(path):
                    raise FileNotFoundError(path)
                libs.append(ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL))
            lib = libs  # type: ignore[assignment]
            _libs[key] = lib
        return _libs[key]


class OracleSim:
    """One simulation held by the port ("port"), by the reference modules ("ref"), or by the
    reference's Solver glue with the GPU Module drop-ins in place of its PreInteraction,
    FluidForce and GravityForce ("gpumod"; `gpu_precision` 0 FP32-pair, 1 FP64)."""

    def __init__(self, params, fields: Dict[str, np.ndarray], kind: str = "port",
                 flavor: str = "strict", threads: Optional[int] = None, gpu_precision: int = 1):
        self.dim = int(params.dim)
        self.kind = kind
        lib = _load(kind, flavor)
        if kind == "port":
            self._lib = lib
            self._pfx = f"orc{self.dim}_"
        else:
            self._lib = lib[self.dim - 1]
            self._pfx = f"ref{self.dim}_"
        self._bind()
        if kind == "gpumod":
            fn = getattr(self._lib, self._pfx + "set_gpu_precision")
            fn.restype = None
            fn.argtypes = [ctypes.c_int]
            fn(int(gpu_precision))
        n = int(np.asarray(fields["mass"]).shape[0])
        self.n = n
        cp = params.to_c(OrcParams)
        if threads:
            self._f("set_threads")(int(threads))
        self._h = self._f("create")(ctypes.byref(cp), n)
        if not self._h:
            raise RuntimeError("oracle create failed")
        for name, arr in fields.items():
            if name in FIELD_ID:
                self.set(name, arr)

    def _bind(self):
        L, p = self._lib, self._pfx
        sigs = {
            "create": (ctypes.c_void_p, [ctypes.POINTER(OrcParams), ctypes.c_int]),
            "destroy": (None, [ctypes.c_void_p]),
            "set_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
            "get_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
            "set_scalar": (None, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]),
            "get_scalar": (ctypes.c_double, [ctypes.c_void_p, ctypes.c_int]),
            "initialize": (ctypes.c_int, [ctypes.c_void_p]),
            "stage": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
            "step": (ctypes.c_int, [ctypes.c_void_p]),
            "neighbors": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
            "tree_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
            "energy": (None, [ctypes.c_void_p, ctypes.c_void_p]),
            "newton_failures": (ctypes.c_int, [ctypes.c_void_p]),
            "set_threads": (None, [ctypes.c_int]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, p + name)
            fn.restype = res
            fn.argtypes = args

    def _f(self, name):
        return getattr(self._lib, self._pfx + name)

    def width(self, name: str) -> int:
        if name in VECTOR:
            return self.dim
        if name == "grad_v":
            return self.dim * self.dim
        return 1

    def set(self, name: str, arr) -> None:
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).reshape(self.n, -1))
        if a.shape[1] != self.width(name):
            raise ValueError(f"{name}: expected width {self.width(name)}, got {a.shape[1]}")
        rc = self._f("set_field")(self._h, FIELD_ID[name], a.ctypes.data)
        if rc:
            raise RuntimeError(f"set_field({name}) -> {rc}")

    def get(self, name: str) -> np.ndarray:
        w = self.width(name)
        a = np.empty((self.n, w), dtype=np.float64)
        rc = self._f("get_field")(self._h, FIELD_ID[name], a.ctypes.data)
        if rc:
            raise RuntimeError(f"get_field({name}) -> {rc}")
        return a[:, 0].copy() if (w == 1 and name not in VECTOR) else a

    def scalar(self, which: str) -> float:
        return self._f("get_scalar")(self._h, {"time": 0, "dt": 1, "h_per_v_sig": 2}[which])

    def set_scalar(self, which: str, v: float) -> None:
        self._f("set_scalar")(self._h, {"time": 0, "dt": 1, "h_per_v_sig": 2}[which], float(v))

    def _error(self, what: str, rc: int) -> RuntimeError:
        text = ""
        if self.kind != "port":
            fn = getattr(self._lib, self._pfx + "last_exception")
            fn.restype = ctypes.c_char_p
            fn.argtypes = []
            text = ": " + fn().decode(errors="replace")
        return RuntimeError(f"{what} -> {rc}{text}")

    def initialize(self) -> None:
        rc = self._f("initialize")(self._h)
        if rc:
            raise self._error("initialize", rc)

    def stage(self, name: str) -> None:
        rc = self._f("stage")(self._h, STAGES[name])
        if rc:
            raise self._error(f"stage {name}", rc)

    def step(self) -> None:
        rc = self._f("step")(self._h)
        if rc:
            raise self._error("step", rc)

    def neighbors(self, is_ij: bool, exhaustive: bool = False, cap: Optional[int] = None,
                  counts_only: bool = False):
        """Neighbour counts and lists (rows of `cap` ids, the first count entries valid) for the
        current smoothing lengths; with counts_only the lists are not stored (list is None)."""
        cap = cap or 2048
        counts = np.zeros(self.n, dtype=np.int32)
        lst = None if counts_only else np.zeros((self.n, cap), dtype=np.int32)
        rc = self._f("neighbors")(self._h, int(is_ij), int(exhaustive), counts.ctypes.data,
                                  None if lst is None else lst.ctypes.data, cap)
        if rc:
            raise RuntimeError(f"neighbors -> {rc}")
        return counts, lst

    def tree_stats(self) -> np.ndarray:
        out = np.zeros(130, dtype=np.int32)
        self._f("tree_stats")(self._h, out.ctypes.data)
        return out

    def energy(self) -> np.ndarray:
        out = np.zeros(4 + self.dim)
        self._f("energy")(self._h, out.ctypes.data)
        return out

    def newton_failures(self) -> int:
        return int(self._f("newton_failures")(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._f("destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
