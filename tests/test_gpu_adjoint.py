"""The device adjoint (sphgpu_adjoint_step / sphgpu_adjoint_initialize behind
sphcode_gb300.adjoint.SphRunFunction) on the Gresho-Chan vortex (standard SPH and the
pressure-energy form, cubic spline, periodic [-0.5, 0.5]^2, gamma 5/3), loss
L = sum (rho_final - 1)^2.

- against an independent host adjoint (tests/adjoint_check.cpp: all pairs, Newton to round-off)
  on a 16 x 16 lattice;
- against central finite differences of the FP64 forward pass, at the relative tolerance 1e-4,
  in the initial internal energy, avAlpha and the initial velocities.  The velocity direction is
  taken on the vortex with a small velocity perturbation: in the vortex itself the rigid core and
  the gas at rest have v_ij . r_ij = 0 exactly for every pair, which puts the viscosity switch
  (v_ij . r_ij < 0) on its kink, and a central difference there averages two one-sided slopes;
- FP32-pair adjoint against the FP64 adjoint, at the stated tolerance;
- the checkpoint interval changes nothing (the recomputation is deterministic).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))

FD_TOL = 1e-4
FP32_FIELD_TOL = 5e-2     # max |g32 - g64| / max |g64| over the gradient field
FP32_DIR_TOL = 2e-2       # directional derivative along a random direction
FP32_ALPHA_TOL = 1e-3


def gresho(n_side, noise=0.0, seed=3, sph_type="ssph"):
    from sphcode_gb300 import ics
    p, f = ics.gresho(n_side)
    p.sph_type = sph_type
    if noise:
        rng = np.random.default_rng(seed)
        f["vel"] = f["vel"] + noise * rng.standard_normal(f["vel"].shape)
    return p, f


def gradients(run, f, p):
    import torch
    from sphcode_gb300.adjoint import density_misfit
    v0 = torch.tensor(f["vel"], device="cuda", requires_grad=True)
    u0 = torch.tensor(f["ene"], device="cuda", requires_grad=True)
    al = torch.tensor(p.av_alpha, dtype=torch.float64, device="cuda", requires_grad=True)
    L = density_misfit(run, v0, u0, al)
    L.backward()
    return (float(L.detach()), v0.grad.detach().cpu().numpy(), u0.grad.detach().cpu().numpy(),
            float(al.grad.detach()))


def loss(run, v, u, alpha):
    import torch
    rho = run.forward(torch.tensor(v, device="cuda"), torch.tensor(u, device="cuda"), alpha, keep=False)
    return float(((rho - 1.0) ** 2).sum())


@pytest.fixture(scope="module")
def host_adjoint(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("adjh") / "libadjcheck.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC",
                           os.path.join(HERE, "adjoint_check.cpp"), "-o", out])
    lib = ctypes.CDLL(out)
    P = ctypes.c_void_p
    lib.adj_gradient.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int, P, P, P, P, P, P, P]
    return lib


@pytest.mark.parametrize("sph_type", ["ssph", "disph"])
@pytest.mark.parametrize("noise", [0.01, 0.05])
def test_adjoint_matches_host(gpu_lib, host_adjoint, noise, sph_type):
    """Velocity noise keeps every pair off v_ij . r_ij = 0 (see the module docstring), where the
    two sides may legitimately take different branches on round-off."""
    from sphcode_gb300.adjoint import SphRun
    p, f = gresho(16, noise, sph_type=sph_type)
    steps = 5
    run = SphRun(p, f, steps, precision="fp64", checkpoint_every=2)
    L, gv, gu, ga = gradients(run, f, p)
    run.close()
    n = f["mass"].size
    x = np.ascontiguousarray(f["pos"].reshape(-1))
    v = np.ascontiguousarray(f["vel"].reshape(-1))
    u = np.ascontiguousarray(f["ene"])
    hv, hu, hr = np.zeros(2 * n), np.zeros(n), np.zeros(n)
    ha = ctypes.c_double()
    host_adjoint.adj_gradient(0, 0 if sph_type == "ssph" else 1, n, steps, run.dt, p.av_alpha,
                              float(p.neighbor_number), 1,
                              x.ctypes.data, v.ctypes.data, u.ctypes.data, hv.ctypes.data, hu.ctypes.data,
                              ctypes.addressof(ha), hr.ctypes.data)
    # the device smoothing lengths are the reference's Newton iterates (converged to a relative
    # step below 2e-4, i.e. to ~1e-8 after the last quadratic step), the host's are exact roots
    errs = {
        "loss": abs(L - float(((hr - 1.0) ** 2).sum())) / L,
        "vbar": np.abs(gv.reshape(-1) - hv).max() / np.abs(hv).max(),
        "ubar": np.abs(gu - hu).max() / np.abs(hu).max(),
        "alpha_bar": abs(ga - ha.value) / max(abs(ha.value), 1e-300),
    }
    assert errs["loss"] <= 1e-6, errs
    assert max(errs["vbar"], errs["ubar"]) <= 1e-5, errs
    assert errs["alpha_bar"] <= 1e-5 or abs(ga - ha.value) <= 1e-9 * np.abs(hv).max(), errs


@pytest.fixture(scope="module", params=["ssph", "disph"])
def fd_case(gpu_lib, request):
    from sphcode_gb300.adjoint import SphRun
    p, f = gresho(64, 0.05, sph_type=request.param)
    run = SphRun(p, f, 30, precision="fp64", checkpoint_every=20)
    res = gradients(run, f, p)
    yield p, f, run, res
    run.close()


def test_finite_differences(fd_case):
    p, f, run, (L, gv, gu, ga) = fd_case
    rng = np.random.default_rng(11)
    # velocity: along the gradient (largest signal against the smoothing-length iterates' own
    # convergence tolerance, which moves the loss by tiny steps when an iteration count changes)
    dv = gv / np.abs(gv).max()
    du = rng.standard_normal(f["ene"].shape)
    eps = 1e-6
    fv = (loss(run, f["vel"] + eps * dv, f["ene"], p.av_alpha)
          - loss(run, f["vel"] - eps * dv, f["ene"], p.av_alpha)) / (2 * eps)
    fu = (loss(run, f["vel"], f["ene"] + eps * du, p.av_alpha)
          - loss(run, f["vel"], f["ene"] - eps * du, p.av_alpha)) / (2 * eps)
    fa = (loss(run, f["vel"], f["ene"], p.av_alpha + eps)
          - loss(run, f["vel"], f["ene"], p.av_alpha - eps)) / (2 * eps)
    errs = {"v": abs(float((gv * dv).sum()) - fv) / abs(fv), "u": abs(float((gu * du).sum()) - fu) / abs(fu),
            "alpha": abs(ga - fa) / abs(fa)}
    assert max(errs.values()) <= FD_TOL, errs


def test_fp32_adjoint_against_fp64(fd_case):
    from sphcode_gb300.adjoint import SphRun
    p, f, run64, (L, gv, gu, ga) = fd_case
    run = SphRun(p, f, 30, dt=run64.dt, precision="fp32", checkpoint_every=20)
    L32, gv32, gu32, ga32 = gradients(run, f, p)
    run.close()
    rng = np.random.default_rng(5)
    dv = rng.standard_normal(f["vel"].shape)
    d64 = float((gv * dv).sum())
    errs = {"loss": abs(L32 - L) / L, "vbar": np.abs(gv32 - gv).max() / np.abs(gv).max(),
            "ubar": np.abs(gu32 - gu).max() / np.abs(gu).max(),
            "dir": abs(float((gv32 * dv).sum()) - d64) / abs(d64), "alpha": abs(ga32 - ga) / abs(ga)}
    assert errs["loss"] <= 1e-3, errs
    assert max(errs["vbar"], errs["ubar"]) <= FP32_FIELD_TOL, errs
    assert errs["dir"] <= FP32_DIR_TOL, errs
    assert errs["alpha"] <= FP32_ALPHA_TOL, errs


def test_checkpoint_interval_is_invisible(gpu_lib):
    from sphcode_gb300.adjoint import SphRun
    p, f = gresho(32, 0.05)
    out = []
    for k in (1, 4, 20):
        run = SphRun(p, f, 9, dt=1e-3, precision="fp64", checkpoint_every=k)
        out.append(gradients(run, f, p))
        run.close()
    for o in out[1:]:
        assert o[0] == out[0][0]
        assert np.array_equal(o[1], out[0][1])
        assert np.array_equal(o[2], out[0][2])
        assert o[3] == out[0][3]
