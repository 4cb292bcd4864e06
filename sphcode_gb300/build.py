"""In-tree build of the sphgpu CUDA library (sm_103a) and its C-ABI.

``build_library()`` compiles every ``csrc/*.cu`` translation unit with nvcc in parallel and links
``sphcode_gb300/_lib/libsphgpu.so``.  Objects are rebuilt only when a source or header is newer
than the object.  No CMake and no torch extension machinery: the library is a plain shared object
with ``extern "C"`` entry points (include/sphgpu.h), loaded with ctypes.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsphgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
# The integrator and the tree keys restate FP64 arithmetic of the reference operation by
# operation; without contraction into FMAs their results are bit-identical to it.
NO_FMA = {"integrate.cu", "tree.cu"}
# The pair kernels take FP32 division and square root from the fast hardware approximations:
# every membership decision is made on products and sums only (and re-decided in FP64 inside its
# guard band), so only the FP32 pair terms see the approximation.  FP64 arithmetic is unaffected.
FAST_F32 = {"pre_d1.cu", "pre_d2.cu", "pre_d3.cu", "fluid_d1.cu", "fluid_d2.cu", "fluid_d3.cu",
            "gravity.cu", "neighbors.cu", "adjoint_d1.cu", "adjoint_d2.cu", "adjoint_d3.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> List[str]:
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(target: str, deps: List[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, jobs: int = 0, verbose: bool = False) -> str:
    """Compile and link the library; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    exe = nvcc()
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            flags = list(COMMON)
            if os.path.basename(s) in NO_FMA:
                flags.append("--fmad=false")
            if os.path.basename(s) in FAST_F32:
                flags += ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
            todo.append([exe, *ARCH, *flags, "-c", s, "-o", o])

    def run(cmd):
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + p.stdout)
        if verbose and p.stdout.strip():
            print(p.stdout)
        return p.stdout

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(run, todo))
    if force or todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        run([exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True))
