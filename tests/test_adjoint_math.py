"""The adjoint algebra of the device adjoint (sphcode_gb300/csrc/adjoint_math.cuh), built for the
host into an all-pairs 2D periodic SPH run (tests/adjoint_check.cpp; standard form and
pressure-energy form) and checked against central finite differences of the same forward map.

Single evaluation: the gradient of a random linear functional of (a, du/dt, rho) after one
PreInteraction + FluidForce, in x, v and u, with the smoothing length as the exact Newton root.
Multi-step: the gradient of L = sum (rho_final - 1)^2 after the kick-drift-kick leapfrog, in the
initial v, the initial u and avAlpha.  The multi-step cases add velocity noise to the vortex: in a
rigid rotation (and in gas at rest) v_ij . r_ij = 0 for every pair, which puts the viscosity's
v_ij . r_ij < 0 switch exactly on its kink, where a central difference averages the two one-sided
slopes and no derivative exists."""
import ctypes
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("adj") / "libadjcheck.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC",
                           os.path.join(HERE, "adjoint_check.cpp"), "-o", out])
    lb = ctypes.CDLL(out)
    lb.adj_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                             ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    lb.adj_check_single.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    return lb


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("sph_type", [0, 1])
@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("balsara", [0, 1])
@pytest.mark.parametrize("which", [1, 2, 4])
def test_single_evaluation(lib, sph_type, kernel, balsara, which):
    out = (ctypes.c_double * 7)()
    lib.adj_check_single(kernel, sph_type, 10, 1e-6, balsara, which, out)
    # the fused forms of the device passes equal the two-call forms
    assert out[6] <= 1e-12, out[6]
    for k, name in enumerate(("x", "v", "u")):
        adj, fd = out[2 * k], out[2 * k + 1]
        if fd == 0.0:
            assert adj == 0.0, name
            continue
        assert rel(adj, fd) < 1e-6, (name, adj, fd)


@pytest.mark.parametrize("sph_type", [0, 1])
@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("balsara", [0, 1])
def test_leapfrog_steps(lib, sph_type, kernel, balsara):
    out = (ctypes.c_double * 7)()
    lib.adj_check(kernel, sph_type, 10, 3, 1e-5, balsara, 0.5, out)
    assert rel(out[0], out[1]) < 1e-6, ("v", out[0], out[1])
    assert rel(out[2], out[3]) < 5e-5, ("u", out[2], out[3])
    assert rel(out[4], out[5]) < 5e-5, ("alpha", out[4], out[5])
