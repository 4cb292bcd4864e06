"""ctypes binding of the sphgpu C-ABI (include/sphgpu.h) and a device-resident simulation handle.

This is the product path: every call goes to the CUDA library ``_lib/libsphgpu.so`` built from
``csrc/`` for sm_103a.  There is no CPU fallback; if the library is missing or no GPU is present
the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import re
import threading
from typing import Dict, Iterable, List, Optional, Sequence

import numpy as np

from .params import CParams, SPHParameters

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsphgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "sphgpu.h")

FIELDS = ["pos", "vel", "vel_p", "acc", "mass", "dens", "pres", "ene", "ene_p", "dene", "sml",
          "sound", "balsara", "alpha", "gradh", "phi", "neighbor", "grad_d", "grad_p", "grad_v"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
VECTOR = {"pos", "vel", "vel_p", "acc", "grad_d", "grad_p"}
PRECISION = {"fp32": 0, "fp32_pair": 0, "fp64": 1}

STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NODE_POOL", 4: "ERR_CAPACITY",
          5: "ERR_NOT_FINITE", 6: "ERR_STATE", 7: "ERR_NO_DEVICE"}

TUNING = {"group_warps": 0, "fluid_warps": 1, "gravity_warps": 2, "tile_cap": 3, "autotune": 4,
          "timing": 5, "graph": 6, "graph_kernels": 7, "overflow_pre": 8, "overflow_fluid": 9,
          "tile_cap_pre": 10, "tune_rejects": 11, "pass2_scale": 12, "fixed_dt": 18, "aos_reuse": 19,
          "tree_levels": 20, "depth_cap": 21, "tile_limit": 22, "node_limit": 23,
          "tune_fail_mask": 24, "count_work": 25, "leaf_cap1": 27, "pair_sched": 28, "bulk_stage": 29,
          "group_rule": 30, "prewalk": 31, "fused_levels": 32,
          "inject_barrier_timeout": 33, "key_table": 34, "gravity_items": 35}


class SphGpuError(RuntimeError):
    """A non-zero sphgpu_status; ``code`` holds the status, the message the library's text."""

    def __init__(self, code: int, where: str, text: str):
        self.code = code
        super().__init__(f"{where}: {STATUS.get(code, code)}: {text}")


class AosLayout(ctypes.Structure):
    """sphgpu_aos_layout."""
    _fields_ = [("stride", ctypes.c_size_t)] + [
        (n, ctypes.c_long) for n in ("pos", "vel", "vel_p", "acc", "mass", "dens", "pres", "ene",
                                     "ene_p", "dene", "sml", "sound", "balsara", "alpha", "gradh",
                                     "phi", "neighbor")]


_lock = threading.Lock()
_lib: Optional[ctypes.CDLL] = None

_P = ctypes.c_void_p
_SIGS = {
    "sphgpu_create": (ctypes.c_int, [ctypes.POINTER(CParams), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "sphgpu_create_batch": (ctypes.c_int, [ctypes.POINTER(CParams), ctypes.c_int, ctypes.c_int, _P, ctypes.c_int, ctypes.POINTER(_P)]),
    "sphgpu_destroy": (ctypes.c_int, [_P]),
    "sphgpu_set_field": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "sphgpu_get_field": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "sphgpu_upload_aos": (ctypes.c_int, [_P, _P, ctypes.POINTER(AosLayout)]),
    "sphgpu_download_aos": (ctypes.c_int, [_P, _P, ctypes.POINTER(AosLayout)]),
    "sphgpu_set_scalar": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    "sphgpu_get_scalar": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "sphgpu_make_tree": (ctypes.c_int, [_P]),
    "sphgpu_pre_interaction": (ctypes.c_int, [_P]),
    "sphgpu_fluid_force": (ctypes.c_int, [_P]),
    "sphgpu_gravity_force": (ctypes.c_int, [_P]),
    "sphgpu_timestep": (ctypes.c_int, [_P]),
    "sphgpu_predict": (ctypes.c_int, [_P]),
    "sphgpu_correct": (ctypes.c_int, [_P]),
    "sphgpu_initialize": (ctypes.c_int, [_P]),
    "sphgpu_step": (ctypes.c_int, [_P, ctypes.c_int]),
    "sphgpu_synchronize": (ctypes.c_int, [_P]),
    "sphgpu_neighbors": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, ctypes.c_int]),
    "sphgpu_energy": (ctypes.c_int, [_P, ctypes.c_int, _P]),
    "sphgpu_tree_stats": (ctypes.c_int, [_P, _P]),
    "sphgpu_target_groups": (ctypes.c_int, [_P, _P, _P]),
    "sphgpu_newton_failures": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "sphgpu_last_error": (ctypes.c_char_p, [_P]),
    "sphgpu_set_tuning": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "sphgpu_get_tuning": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "sphgpu_stage_times": (ctypes.c_int, [_P, _P]),
    "sphgpu_pair_counters": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "sphgpu_bench_steps": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "sphgpu_measure_peaks": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "sphgpu_energy_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _P, _P, _P, _P, _P, _P]),
    "sphgpu_get_state": (ctypes.c_int, [_P, _P]),
    "sphgpu_set_state": (ctypes.c_int, [_P, _P]),
    "sphgpu_adjoint_step": (ctypes.c_int, [_P, _P, _P, _P]),
    "sphgpu_adjoint_initialize": (ctypes.c_int, [_P, _P, _P, _P]),
}


def measure_peaks():
    """(FP32, FP64) FMA throughput of the current device in TFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(library().sphgpu_measure_peaks(ctypes.byref(a), ctypes.byref(b)), "measure_peaks")
    return a.value, b.value


def header_functions(path: str = HEADER) -> List[str]:
    """Names of the functions include/sphgpu.h declares."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sphgpu_[a-z_0-9]+)\s*\(", text)))


def library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load (once) and bind the CUDA library.  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise FileNotFoundError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def _check(rc: int, where: str, handle=None) -> None:
    if rc != 0:
        lib = library()
        msg = lib.sphgpu_last_error(handle)
        raise SphGpuError(rc, where, msg.decode() if msg else "")


class GpuSimulation:
    """One simulation (or a batch of independent runs) resident on the current CUDA device.

    ``fields`` maps field names to float64 arrays in particle order (vector fields ``(N, DIM)``).
    ``runs`` (optional) lists the particle counts of independent runs stored back to back.
    """

    def __init__(self, params: SPHParameters, fields: Dict[str, np.ndarray], precision: str = "fp32",
                 runs: Optional[Sequence[int]] = None):
        lib = library()
        self.lib = lib
        self.params = params
        self.dim = int(params.dim)
        self.precision = precision
        n = int(np.asarray(fields["mass"]).shape[0])
        self.n = n
        cp = params.to_c(CParams)
        h = _P()
        if runs is None:
            rc = lib.sphgpu_create(ctypes.byref(cp), self.dim, n, PRECISION[precision], ctypes.byref(h))
            self.n_runs = 1
        else:
            sizes = np.ascontiguousarray(np.asarray(runs, dtype=np.int32))
            if int(sizes.sum()) != n:
                raise ValueError("run sizes do not add up to the particle count")
            rc = lib.sphgpu_create_batch(ctypes.byref(cp), self.dim, int(sizes.size), sizes.ctypes.data,
                                         PRECISION[precision], ctypes.byref(h))
            self.n_runs = int(sizes.size)
        _check(rc, "sphgpu_create")
        self._h = h
        for name, arr in fields.items():
            if name in FIELD_ID:
                self.set(name, arr)

    # ---- fields -----------------------------------------------------------------------------
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
        _check(self.lib.sphgpu_set_field(self._h, FIELD_ID[name], a.ctypes.data), f"set {name}", self._h)

    def get(self, name: str) -> np.ndarray:
        w = self.width(name)
        a = np.empty((self.n, w), dtype=np.float64)
        _check(self.lib.sphgpu_get_field(self._h, FIELD_ID[name], a.ctypes.data), f"get {name}", self._h)
        return a[:, 0].copy() if (w == 1 and name not in VECTOR) else a

    def scalar(self, which: str, run: int = 0) -> float:
        v = ctypes.c_double()
        _check(self.lib.sphgpu_get_scalar(self._h, {"time": 0, "dt": 1, "h_per_v_sig": 2}[which], run,
                                          ctypes.byref(v)), "get_scalar", self._h)
        return v.value

    def set_scalar(self, which: str, value: float, run: int = 0) -> None:
        _check(self.lib.sphgpu_set_scalar(self._h, {"time": 0, "dt": 1, "h_per_v_sig": 2}[which], run,
                                          float(value)), "set_scalar", self._h)

    # ---- integrator state and adjoint (device pointers, caller order) -------------------------
    def state_size(self) -> int:
        """Doubles of the state vector [x | v | u | a | du/dt | rho]."""
        return self.n * (3 * self.dim + 3)

    def adjoint_size(self) -> int:
        """Doubles of the adjoint vector [xbar | vbar | ubar | abar | dubar]."""
        return self.n * (3 * self.dim + 2)

    def get_state(self, dev_ptr: int) -> None:
        _check(self.lib.sphgpu_get_state(self._h, _P(dev_ptr)), "get_state", self._h)

    def set_state(self, dev_ptr: int) -> None:
        _check(self.lib.sphgpu_set_state(self._h, _P(dev_ptr)), "set_state", self._h)

    def adjoint_step(self, adj_ptr: int, dens_bar_ptr: int, alpha_bar_ptr: int) -> None:
        _check(self.lib.sphgpu_adjoint_step(self._h, _P(adj_ptr), _P(dens_bar_ptr or None), _P(alpha_bar_ptr)),
               "adjoint_step", self._h)

    def adjoint_initialize(self, adj_ptr: int, dens_bar_ptr: int, alpha_bar_ptr: int) -> None:
        _check(self.lib.sphgpu_adjoint_initialize(self._h, _P(adj_ptr), _P(dens_bar_ptr or None),
                                                  _P(alpha_bar_ptr)), "adjoint_initialize", self._h)

    # ---- stages -----------------------------------------------------------------------------
    def initialize(self) -> None:
        _check(self.lib.sphgpu_initialize(self._h), "initialize", self._h)

    def step(self, n: int = 1) -> None:
        _check(self.lib.sphgpu_step(self._h, int(n)), "step", self._h)

    def make_tree(self) -> None:
        _check(self.lib.sphgpu_make_tree(self._h), "make_tree", self._h)

    def pre_interaction(self) -> None:
        _check(self.lib.sphgpu_pre_interaction(self._h), "pre_interaction", self._h)

    def fluid_force(self) -> None:
        _check(self.lib.sphgpu_fluid_force(self._h), "fluid_force", self._h)

    def gravity_force(self) -> None:
        _check(self.lib.sphgpu_gravity_force(self._h), "gravity_force", self._h)

    def timestep(self) -> None:
        _check(self.lib.sphgpu_timestep(self._h), "timestep", self._h)

    def predict(self) -> None:
        _check(self.lib.sphgpu_predict(self._h), "predict", self._h)

    def correct(self) -> None:
        _check(self.lib.sphgpu_correct(self._h), "correct", self._h)

    def synchronize(self) -> None:
        _check(self.lib.sphgpu_synchronize(self._h), "synchronize", self._h)

    # ---- diagnostics ------------------------------------------------------------------------
    def neighbor_counts(self, is_ij: bool) -> np.ndarray:
        counts = np.zeros(self.n, dtype=np.int32)
        _check(self.lib.sphgpu_neighbors(self._h, int(is_ij), counts.ctypes.data, None, 0),
               "neighbors", self._h)
        return counts

    def bench_steps(self, n: int, flush_l2: bool = True) -> float:
        """Device milliseconds of n steps (CUDA events on the library's stream, L2 flushed
        between steps outside the timed brackets)."""
        ms = ctypes.c_double()
        _check(self.lib.sphgpu_bench_steps(self._h, int(n), int(flush_l2), ctypes.byref(ms)),
               "bench_steps", self._h)
        return ms.value

    def neighbors(self, is_ij: bool, cap: int = 1024):
        """Neighbour counts and lists (cap ids per particle) for the current smoothing lengths,
        in the caller's order; cap = 0 returns the counts only (lists None)."""
        counts = np.zeros(self.n, dtype=np.int32)
        lst = np.zeros((self.n, cap), dtype=np.int32) if cap > 0 else None
        _check(self.lib.sphgpu_neighbors(self._h, int(is_ij), counts.ctypes.data,
                                         None if lst is None else lst.ctypes.data, int(cap)),
               "neighbors", self._h)
        return counts, lst

    def energy(self, run: int = 0) -> np.ndarray:
        out = np.zeros(4 + self.dim)
        _check(self.lib.sphgpu_energy(self._h, run, out.ctypes.data), "energy", self._h)
        return out

    def target_groups(self):
        """Group index of every particle (caller order) in the pair kernels' group list of the
        last tree build, and the number of groups."""
        g = np.zeros(self.n, dtype=np.int32)
        ng = ctypes.c_int()
        _check(self.lib.sphgpu_target_groups(self._h, g.ctypes.data, ctypes.byref(ng)), "target_groups", self._h)
        return g, ng.value

    def tree_stats(self) -> np.ndarray:
        out = np.zeros(130, dtype=np.int32)
        _check(self.lib.sphgpu_tree_stats(self._h, out.ctypes.data), "tree_stats", self._h)
        return out

    def newton_failures(self) -> int:
        v = ctypes.c_int()
        _check(self.lib.sphgpu_newton_failures(self._h, ctypes.byref(v)), "newton_failures", self._h)
        return v.value

    def set_tuning(self, which: str, value: int) -> None:
        _check(self.lib.sphgpu_set_tuning(self._h, TUNING[which], int(value)), "set_tuning", self._h)

    def get_tuning(self, which: str) -> int:
        v = ctypes.c_int()
        _check(self.lib.sphgpu_get_tuning(self._h, TUNING[which], ctypes.byref(v)), "get_tuning", self._h)
        return v.value

    def fail_range(self) -> List[int]:
        """The last target range no pair-kernel pass could fit: [first particle (key order),
        count, search radius x 1e9, leaves, overflow code] (tuning knobs 13..17)."""
        out = []
        for which in range(13, 18):
            v = ctypes.c_int()
            _check(self.lib.sphgpu_get_tuning(self._h, which, ctypes.byref(v)), "get_tuning", self._h)
            out.append(v.value)
        return out

    def stage_times(self) -> Dict[str, float]:
        out = np.zeros(5)
        _check(self.lib.sphgpu_stage_times(self._h, out.ctypes.data), "stage_times", self._h)
        return dict(zip(["tree", "pre", "fluid", "gravity", "integrate"], out.tolist()))

    COUNTERS = ["pre_targets", "pre_candidates", "pre_iters", "pre_iter_pairs", "pre_pairs",
                "pre_tests", "fluid_tests", "pre_groups", "fluid_groups", "grav_nodes", "grav_pairs"]

    def pair_counters(self, reset: bool = True) -> Dict[str, int]:
        """Work counters of the pair kernels collected while the count_work knob is on."""
        out = np.zeros(16, dtype=np.uint64)
        _check(self.lib.sphgpu_pair_counters(self._h, out.ctypes.data, int(reset)), "pair_counters", self._h)
        return {k: int(v) for k, v in zip(self.COUNTERS, out.tolist())}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.sphgpu_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
