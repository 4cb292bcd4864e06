"""Gradient harness: the device adjoint of a standard-SPH run behind ``torch.autograd.Function``.

PyTorch is only the harness here (device buffers and the autograd interface): the forward run is
the library's own step (one CUDA graph per step) and the backward pass is the library's
hand-written adjoint kernels (sphgpu_adjoint_step / sphgpu_adjoint_initialize), reached through
the C-ABI.

A run is Solver::initialize followed by ``steps`` Solver::integrate steps (src/solver.cpp:
392-474) with a fixed dt.  The forward pass keeps the integrator state every
``checkpoint_every`` steps; the backward pass walks the segments in reverse, recomputes the
states of a segment from its checkpoint, and reverses its steps one by one, so the memory held
is O(n (steps / k + k)) states instead of O(n steps).
"""
from __future__ import annotations

import copy
import time
from typing import Dict, Optional

import numpy as np
import torch

from .params import SPHParameters
from .sphgpu import GpuSimulation


class SphRun:
    """A fixed-dt run, differentiable in the initial velocities, the initial internal energy and
    avAlpha.  ``fields`` are the initial fields (pos, vel, mass, dens, ene; caller order)."""

    def __init__(self, param: SPHParameters, fields: Dict[str, np.ndarray], steps: int,
                 dt: Optional[float] = None, precision: str = "fp64", checkpoint_every: int = 20,
                 device: str = "cuda"):
        if checkpoint_every < 1:
            raise ValueError("checkpoint_every must be >= 1")
        self.param = param
        self.fields = {k: np.asarray(v, dtype=np.float64) for k, v in fields.items()}
        self.steps = int(steps)
        self.k = int(checkpoint_every)
        self.precision = precision
        self.device = torch.device(device)
        self.dim = int(param.dim)
        self.n = int(self.fields["mass"].shape[0])
        self._sim: Optional[GpuSimulation] = None
        self._alpha: Optional[float] = None
        if dt is None:
            # the CFL step of the initial state (TimeStep, src/timestep.cpp:18-38), then held fixed
            sim = self._simulation(param.av_alpha)
            sim.initialize()
            sim.timestep()
            dt = sim.scalar("dt")
        self.dt = float(dt)
        self.timings: Dict[str, float] = {}

    # ---- device simulation -------------------------------------------------------------------
    def _simulation(self, alpha: float) -> GpuSimulation:
        if self._sim is None or self._alpha != alpha:
            if self._sim is not None:
                self._sim.close()
            p = copy.deepcopy(self.param)
            p.av_alpha = float(alpha)
            sim = GpuSimulation(p, self.fields, precision=self.precision)
            sim.set_tuning("autotune", 0)
            sim.set_tuning("fixed_dt", 1)
            self._sim, self._alpha = sim, alpha
        return self._sim

    def _state_tensor(self) -> torch.Tensor:
        return torch.empty(self.n * (3 * self.dim + 3), dtype=torch.float64, device=self.device)

    def initial_state(self, v0: torch.Tensor, u0: torch.Tensor) -> torch.Tensor:
        """[x | v | u | a | du/dt | rho] of the initial fields with the given v and u."""
        n, d = self.n, self.dim
        s = torch.zeros(n * (3 * d + 3), dtype=torch.float64, device=self.device)
        s[: n * d] = torch.as_tensor(self.fields["pos"].reshape(-1), device=self.device)
        s[n * d: 2 * n * d] = v0.detach().reshape(-1).to(self.device, torch.float64)
        s[2 * n * d: 2 * n * d + n] = u0.detach().reshape(-1).to(self.device, torch.float64)
        s[3 * n * d + 2 * n:] = torch.as_tensor(self.fields["dens"].reshape(-1), device=self.device)
        return s

    def density(self, state: torch.Tensor) -> torch.Tensor:
        return state[-self.n:]

    # ---- forward / backward ------------------------------------------------------------------
    def forward(self, v0: torch.Tensor, u0: torch.Tensor, alpha: float, keep: bool = True) -> torch.Tensor:
        """Runs the steps; returns the final density (caller order).  With ``keep`` the
        checkpoints for the backward pass are kept."""
        sim = self._simulation(float(alpha))
        ic = self.initial_state(v0, u0)
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        sim.set_state(ic.data_ptr())
        sim.set_scalar("dt", self.dt)
        sim.initialize()
        sim.set_scalar("dt", self.dt)
        ckpts = []
        done = 0
        while True:
            if keep:
                st = self._state_tensor()
                sim.get_state(st.data_ptr())
                ckpts.append(st)
            if done >= self.steps:
                break
            m = min(self.k, self.steps - done)
            sim.step(m)
            done += m
        final = self._state_tensor() if not keep else ckpts[-1]
        if not keep:
            sim.get_state(final.data_ptr())
        self.timings["forward_s"] = time.perf_counter() - t0
        if keep:
            self._ic, self._ckpts = ic, ckpts[:-1] if self.steps > 0 else []
        return self.density(final).clone()

    def backward(self, dens_bar: torch.Tensor):
        """Reverse sweep; returns (xbar0, vbar0, ubar0, alpha_bar)."""
        sim = self._sim
        n, d = self.n, self.dim
        adj = torch.zeros(n * (3 * d + 2), dtype=torch.float64, device=self.device)
        alpha_bar = torch.zeros(1, dtype=torch.float64, device=self.device)
        dbar = dens_bar.detach().reshape(-1).to(self.device, torch.float64).contiguous()
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        n_seg = len(self._ckpts)
        seg_states = [self._state_tensor() for _ in range(min(self.k, max(self.steps, 1)))]
        for seg in reversed(range(n_seg)):
            t_begin = seg * self.k
            t_end = min(t_begin + self.k, self.steps)
            # recompute the states S_t of the segment from its checkpoint
            sim.set_state(self._ckpts[seg].data_ptr())
            seg_states[0].copy_(self._ckpts[seg])
            torch.cuda.synchronize(self.device)
            for t in range(t_begin + 1, t_end):
                sim.step(1)
                sim.get_state(seg_states[t - t_begin].data_ptr())
            for t in reversed(range(t_begin, t_end)):
                sim.set_state(seg_states[t - t_begin].data_ptr())
                last = t == self.steps - 1
                sim.adjoint_step(adj.data_ptr(), dbar.data_ptr() if last else 0, alpha_bar.data_ptr())
        sim.set_state(self._ic.data_ptr())
        sim.adjoint_initialize(adj.data_ptr(), dbar.data_ptr() if self.steps == 0 else 0, alpha_bar.data_ptr())
        self.timings["backward_s"] = time.perf_counter() - t0
        xbar = adj[: n * d].view(n, d).clone()
        vbar = adj[n * d: 2 * n * d].view(n, d).clone()
        ubar = adj[2 * n * d: 2 * n * d + n].clone()
        return xbar, vbar, ubar, alpha_bar[0].clone()

    def close(self) -> None:
        if self._sim is not None:
            self._sim.close()
            self._sim = None


class SphRunFunction(torch.autograd.Function):
    """final density = F(v0, u0, alpha) for one SphRun; backward through the device adjoint."""

    @staticmethod
    def forward(ctx, v0: torch.Tensor, u0: torch.Tensor, alpha: torch.Tensor, run: SphRun):
        ctx.run = run
        return run.forward(v0, u0, float(alpha))

    @staticmethod
    def backward(ctx, dens_bar: torch.Tensor):
        run: SphRun = ctx.run
        _, vbar, ubar, alpha_bar = run.backward(dens_bar)
        return vbar, ubar, alpha_bar, None


def density_misfit(run: SphRun, v0: torch.Tensor, u0: torch.Tensor, alpha: torch.Tensor,
                   target: float = 1.0) -> torch.Tensor:
    """L = sum (rho_final - target)^2 through the autograd function."""
    rho = SphRunFunction.apply(v0, u0, alpha, run)
    return ((rho - target) ** 2).sum()


def _loss_at(run: SphRun, v: np.ndarray, u: np.ndarray, alpha: float, target: float = 1.0) -> float:
    rho = run.forward(torch.as_tensor(v, device=run.device), torch.as_tensor(u, device=run.device), alpha, keep=False)
    return float(((rho - target) ** 2).sum())


def gradient(run: SphRun, v0: np.ndarray, u0: np.ndarray, alpha: float, target: float = 1.0):
    """(L, dL/dv0, dL/du0, dL/dalpha) of L = sum (rho_final - target)^2 through the autograd
    function."""
    v = torch.tensor(v0, device=run.device, requires_grad=True)
    u = torch.tensor(u0, device=run.device, requires_grad=True)
    a = torch.tensor(float(alpha), dtype=torch.float64, device=run.device, requires_grad=True)
    L = density_misfit(run, v, u, a, target)
    L.backward()
    return float(L.detach()), v.grad.cpu().numpy(), u.grad.cpu().numpy(), float(a.grad)


def finite_difference_check(param: SPHParameters, fields: Dict[str, np.ndarray], steps: int, dt: float,
                            eps: float = 1e-6, checkpoint_every: int = 20) -> Dict[str, float]:
    """Directional derivatives of the FP64 adjoint against central differences of the FP64
    forward pass: along the velocity gradient and the internal-energy gradient themselves
    (scaled to a largest component of 1) and in avAlpha.  Returns the relative differences."""
    run = SphRun(param, fields, steps, dt=dt, precision="fp64", checkpoint_every=checkpoint_every)
    v0, u0, a0 = fields["vel"], fields["ene"], float(param.av_alpha)
    L, gv, gu, ga = gradient(run, v0, u0, a0)
    dv = gv / np.abs(gv).max()
    du = gu / np.abs(gu).max()
    fv = (_loss_at(run, v0 + eps * dv, u0, a0) - _loss_at(run, v0 - eps * dv, u0, a0)) / (2 * eps)
    fu = (_loss_at(run, v0, u0 + eps * du, a0) - _loss_at(run, v0, u0 - eps * du, a0)) / (2 * eps)
    fa = (_loss_at(run, v0, u0, a0 + eps) - _loss_at(run, v0, u0, a0 - eps)) / (2 * eps)
    run.close()
    av, au = float((gv * dv).sum()), float((gu * du).sum())
    return {"loss": L, "v": abs(av - fv) / abs(fv), "u": abs(au - fu) / abs(fu), "alpha": abs(ga - fa) / abs(fa),
            "adjoint": [av, au, ga], "fd": [fv, fu, fa], "eps": eps}


def cost_and_precision(param: SPHParameters, fields: Dict[str, np.ndarray], steps: int, dt: Optional[float] = None,
                       checkpoint_every: int = 20, reps: int = 3) -> Dict[str, object]:
    """Wall time of the forward run (no checkpoints kept) and of the backward sweep (segment
    recomputation + adjoint) in both precisions, and the FP32-pair gradient against FP64."""
    out: Dict[str, object] = {}
    grads = {}
    for prec in ("fp32", "fp64"):
        run = SphRun(param, fields, steps, dt=dt, precision=prec, checkpoint_every=checkpoint_every)
        dt = run.dt
        v0 = torch.as_tensor(fields["vel"], device=run.device)
        u0 = torch.as_tensor(fields["ene"], device=run.device)
        rho = run.forward(v0, u0, param.av_alpha)
        run.backward(2 * (rho - 1))
        tf, tk, tb = [], [], []
        for _ in range(reps):
            run.forward(v0, u0, param.av_alpha, keep=False)
            tf.append(run.timings["forward_s"])
            rho = run.forward(v0, u0, param.av_alpha)
            tk.append(run.timings["forward_s"])
            res = run.backward(2 * (rho - 1))
            tb.append(run.timings["backward_s"])
        grads[prec] = (res[1].cpu().numpy(), res[2].cpu().numpy(), float(res[3]),
                       float(((rho - 1) ** 2).sum()))
        out[prec] = {"forward_s": min(tf), "forward_checkpointed_s": min(tk), "backward_s": min(tb),
                     "backward_over_forward": min(tb) / min(tf)}
        run.close()
    g32, g64 = grads["fp32"], grads["fp64"]
    out["dt"] = dt
    out["fp32_vs_fp64"] = {
        "loss": abs(g32[3] - g64[3]) / g64[3],
        "vbar": float(np.abs(g32[0] - g64[0]).max() / np.abs(g64[0]).max()),
        "ubar": float(np.abs(g32[1] - g64[1]).max() / np.abs(g64[1]).max()),
        "alpha_bar": abs(g32[2] - g64[2]) / abs(g64[2]),
    }
    return out


def perturbation_growth(param: SPHParameters, fields: Dict[str, np.ndarray], steps: int, dt: float,
                        size: float = 1e-12, every: int = 20, seed: int = 7) -> list:
    """max |rho - rho'| every ``every`` steps between the FP64 run and the run whose initial
    velocities carry a random perturbation of the given size: how far a tangent perturbation
    grows, i.e. the horizon over which any gradient of the run is a useful linearisation."""
    run = SphRun(param, fields, every, dt=dt, precision="fp64", checkpoint_every=every)
    sim = run._simulation(float(param.av_alpha))
    out = []
    traj = []
    for pert in (0.0, size):
        v = fields["vel"] + pert * np.random.default_rng(seed).standard_normal(fields["vel"].shape)
        ic = run.initial_state(torch.as_tensor(v), torch.as_tensor(fields["ene"]))
        torch.cuda.synchronize(run.device)
        sim.set_state(ic.data_ptr())
        sim.set_scalar("dt", dt)
        sim.initialize()
        sim.set_scalar("dt", dt)
        rows = []
        for _ in range(steps // every):
            sim.step(every)
            rows.append(sim.get("dens"))
        traj.append(rows)
    for a, b in zip(*traj):
        out.append(float(np.abs(a - b).max()))
    run.close()
    return out
