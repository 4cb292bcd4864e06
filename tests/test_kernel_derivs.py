"""The smoothing-kernel derivatives used by the adjoint kernels (sphcode_gb300/csrc/kderiv.cuh),
built for the host and checked against the reference kernels' published formulas
(include/kernel/cubic_spline.hpp:27-51, include/kernel/wendland_kernel.hpp:30-48) and against
central finite differences, in the manner of the reference's own kernel test
(test/kernel_test/kernel_test.cpp:8-85), here with thresholds."""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def kd(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("kd") / "libkd.so")
    subprocess.check_call(["g++", "-O2", "-std=c++14", "-shared", "-fPIC", "-I",
                           os.path.join(ROOT, "sphcode_gb300", "csrc"),
                           os.path.join(HERE, "kderiv_check.cpp"), "-o", out])
    lib = ctypes.CDLL(out)
    lib.kd_eval.restype = ctypes.c_double
    lib.kd_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
    return lambda D, K, which, r, h: lib.kd_eval(D, K, which, r, h)


def ref_w(D, K, r, h):
    if K == 0:
        s = {1: 2 / 3, 2: 10 / (7 * math.pi), 3: 1 / math.pi}[D]
        hh = 0.5 * h
        q = r / hh
        a, b = max(2 - q, 0.0), max(1 - q, 0.0)
        return s / hh ** D * (0.25 * a ** 3 - b ** 3)
    s = {2: 9 / math.pi, 3: 495 / (32 * math.pi)}[D]
    q = r / h
    a = max(1 - q, 0.0)
    return s / h ** D * a ** 6 * (1 + 6 * q + 35 / 3 * q * q)


def ref_dhw(D, K, r, h):
    if K == 0:
        s = {1: 2 / 3, 2: 10 / (7 * math.pi), 3: 1 / math.pi}[D]
        hh = 0.5 * h
        q = r / hh
        a, b = max(2 - q, 0.0), max(1 - q, 0.0)
        return 0.5 * s / (hh ** D * hh) * (a * a * ((3 + D) * 0.25 * q - 0.5 * D) + b * b * ((-3 - D) * q + D))
    s = {2: 9 / math.pi, 3: 495 / (32 * math.pi)}[D]
    q = r / h
    a = max(1 - q, 0.0)
    return -s / (h ** D * h * 3) * a ** 5 * (3 * D + 15 * D * q + (-56 + 17 * D) * q * q - 35 * (8 + D) * q ** 3)


CASES = [(1, 0), (2, 0), (3, 0), (2, 1), (3, 1)]


@pytest.mark.parametrize("D,K", CASES)
def test_kernel_values_match_reference_formulas(kd, D, K):
    h = 0.37
    for r in np.linspace(0.0, 1.05 * h, 41):
        assert kd(D, K, 0, r, h) == pytest.approx(ref_w(D, K, r, h), rel=1e-12, abs=1e-12)
        assert kd(D, K, 1, r, h) == pytest.approx(ref_dhw(D, K, r, h), rel=1e-11, abs=1e-11)


@pytest.mark.parametrize("D,K", CASES)
def test_derivatives_against_finite_differences(kd, D, K):
    h = 0.37
    eps = 1e-6
    # avoid the piecewise joints q = 1, 2 of the cubic spline and r = 0
    for r in [0.031, 0.09, 0.14, 0.22, 0.27, 0.33]:
        fd_wr = (kd(D, K, 0, r + eps, h) - kd(D, K, 0, r - eps, h)) / (2 * eps)
        assert kd(D, K, 3, r, h) * r == pytest.approx(fd_wr, rel=1e-6, abs=1e-9)          # dW/dr = r F
        fd_wh = (kd(D, K, 0, r, h + eps) - kd(D, K, 0, r, h - eps)) / (2 * eps)
        assert kd(D, K, 1, r, h) == pytest.approx(fd_wh, rel=1e-6, abs=1e-9)
        fd_whh = (kd(D, K, 1, r, h + eps) - kd(D, K, 1, r, h - eps)) / (2 * eps)
        assert kd(D, K, 2, r, h) == pytest.approx(fd_whh, rel=1e-5, abs=1e-7)
        fd_fr = (kd(D, K, 3, r + eps, h) - kd(D, K, 3, r - eps, h)) / (2 * eps)
        assert kd(D, K, 4, r, h) == pytest.approx(fd_fr, rel=1e-5, abs=1e-7)
        fd_fh = (kd(D, K, 3, r, h + eps) - kd(D, K, 3, r, h - eps)) / (2 * eps)
        assert kd(D, K, 5, r, h) == pytest.approx(fd_fh, rel=1e-5, abs=1e-7)
