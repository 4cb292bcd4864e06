"""Benchmark of the SPH particle hot path on one GB300: particle-steps/s.

Default workload: the 2D Kelvin-Helmholtz step, disph + Wendland C4 + artificial conductivity,
786,376 particles (square lattices of spacing 1/1024 in the dense strip and 1/724 outside),
periodic unit box, neighborNumber 64.  One step = TimeStep, predict, octree build, PreInteraction,
FluidForce, (GravityForce), correct, all on the device (Solver::integrate).  Inputs are synthetic
(the seeded/lattice initial conditions of sphcode_gb300/ics.py).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload khi|evrard|gresho|sod]
  python bench.py --impl reference ...   # the reference's own CPU modules on the host cores

Timing: W warm-up steps, then K steps, each bracketed by CUDA events on the library's stream
with a 2 x L2 buffer overwritten between steps outside the brackets; max over ranks.  Under
torchrun every rank runs an independent replica of the workload (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300, FP32-pair vs FP64 form at stated rel err"

# Static flop counts of the reference's pair bodies (each add, multiply, divide and square root
# = 1, an FMA = 2), per pair: FluidForce per interacting pair {r < max(h_i, h_j)}
# (src/fluid_force.cpp:56-116, src/disph/d_fluid_force.cpp:26-86, src/gsph/g_fluid_force.cpp:79-163);
# PreInteraction per Newton iteration and pair {r < h} (src/pre_interaction.cpp:227-283,
# src/disph/d_pre_interaction.cpp:187-217: r_ij, |r_ij|, W, dW/dh, two sums) and per pair of the
# density pass (src/pre_interaction.cpp:78-161, src/disph/d_pre_interaction.cpp:60-154: W, dW/dh,
# the density-type sums, the signal velocity, grad W and the div/rot v sums of Balsara / TD-AV).
FLUID_FLOPS_PER_PAIR = {("disph", 2): 120, ("disph", 3): 135, ("ssph", 2): 110, ("ssph", 3): 125,
                        ("ssph", 1): 90, ("gsph", 1): 180, ("disph", 1): 100}
PRE_NEWTON_FLOPS_PER_PAIR = {1: 44, 2: 47, 3: 50}
PRE_DENS_FLOPS_PER_PAIR = {("disph", 2): 91, ("disph", 3): 110, ("ssph", 2): 86, ("ssph", 3): 104,
                           ("ssph", 1): 60, ("disph", 1): 62, ("gsph", 1): 70}
# Barnes-Hut walk: per leaf pair (HK89-softened potential and force, src/bhtree.cpp:273-299) and per
# accepted monopole (src/bhtree.cpp:327-329).
GRAV_FLOPS_LEAF, GRAV_FLOPS_NODE = 60, 20


# Compulsory HBM bytes of the force stage per particle inside a whole step: FP64 reads of pos(D)
# and sml, the FP32 source records that PreInteraction wrote (48 B), writes of acc(D), dene.
def fluid_bytes_per_particle(D):
    return 8 * (D + 1) + 48 + 8 * (D + 1)


# PreInteraction: reads pos(D), vel(D), mass, dens, ene, alpha, balsara and the FP32 mirrors (32 B
# written and read; the sound speed formed from u), writes sml, dens, pres, gradh, balsara, alpha
# (FP64), the count and FluidForce's FP32 source records (48 B).
def pre_bytes_per_particle(D):
    return 8 * (2 * D + 5) + 32 * 2 + 8 * 6 + 4 + 48


# GravityForce: reads pos(D), mass, sml and the FP32 leaf records (16 B), reads and writes acc(D),
# writes phi; the node records are read from L2.
def grav_bytes_per_particle(D):
    return 8 * (D + 2) + 16 + 16 * D + 8


def aggregate(ms_local, n_local, steps, dist=None, device="cpu"):
    """Whole-job throughput of independent replicas: the slowest rank's time (max over ranks)
    and the particles of all ranks.  Returns (ms_max, particle-steps/s)."""
    if dist is None:
        return ms_local, n_local * steps / (ms_local * 1e-3)
    import torch
    t = torch.tensor([ms_local, float(n_local)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx[:1], op=dist.ReduceOp.MAX)
    dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
    ms = float(mx[0].item())
    return ms, float(t[1].item()) * steps / (ms * 1e-3)


def workload(name):
    """(params, fields, description, run sizes or None)."""
    from sphcode_gb300 import ics
    if name == "ensemble":
        p, f, sizes = ics.ensemble()
        return p, f, "ensemble_1d_gsph2_4096_tubes", sizes
    if name == "khi":
        p, f = ics.khi()
        desc = "khi_2d_disph_wendland_ac"
    elif name == "evrard":
        p, f = ics.evrard()
        desc = "evrard_3d_disph_wendland_balsara_tdav_gravity"
    elif name == "evrard_small":   # 2^18 particles, for profiling captures
        p, f = ics.evrard(1 << 18)
        desc = "evrard_3d_disph_wendland_balsara_tdav_gravity_262144"
    elif name == "gresho":
        p, f = ics.gresho(256)
        desc = "gresho_chan_2d_ssph_cubic"
    elif name == "sod":
        p, f = ics.sod()
        desc = "sod_1d_ssph_cubic"
    else:
        raise SystemExit(f"unknown workload {name}")
    return p, f, desc, None


# ---- clocks --------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.first = 0

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi takes a moment to start: wait for its first sample, so that the samples
            # of the timed region are not lost to its start-up
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def mark(self):
        """The timed region starts: later samples are the ones reported."""
        self.first = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the samples taken from the start of the timed region on (at least the last one)
        lines = self.lines[min(self.first, max(len(self.lines) - 1, 0)):]
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---- reference-layout host particles (SPHParticle, include/particle.hpp:8-33) --------------
def aos_dtype(D):
    fields = [("pos", "f8", (D,)), ("vel", "f8", (D,)), ("vel_p", "f8", (D,)), ("acc", "f8", (D,))]
    fields += [(n, "f8") for n in ("mass", "dens", "pres", "ene", "ene_p", "dene", "sml", "sound",
                                   "balsara", "alpha", "gradh", "phi")]
    fields += [("id", "i4"), ("neighbor", "i4"), ("next", "u8")]
    return np.dtype(fields, align=True)


def aos_layout(dt):
    from sphcode_gb300 import sphgpu
    lay = sphgpu.AosLayout()
    lay.stride = dt.itemsize
    for name in ("pos", "vel", "vel_p", "acc", "mass", "dens", "pres", "ene", "ene_p", "dene", "sml",
                 "sound", "balsara", "alpha", "gradh", "phi", "neighbor"):
        setattr(lay, name, dt.fields[name][1])
    return lay


def pinned_array(nbytes):
    import torch
    t = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    return t, t.numpy()


# ---- CPU baseline / reference arm ------------------------------------------------------------
def cpu_reference_run(name, steps, threads, warmup=0, budget_s=None):
    """Time the reference's own modules (oracle/_ref, built from the reference sources with the
    reference Makefile's flags) or, where they are not built, the C restatement in oracle/, on
    the host cores.  After initialize, `warmup` untimed steps, then up to `steps` timed steps;
    with `budget_s` the timed loop stops once that many seconds have passed (at least one step).
    Returns (particle-steps/s, kind, sample text, seconds, timed steps, warm-up steps)."""
    from oracle import pyoracle
    p, f, desc, runs = workload(name)
    kind = "reference" if pyoracle.reference_available("fast") else "port"
    okind = "ref" if kind == "reference" else "port"
    if runs is not None:
        # the reference runs one tube per process: time the first tubes one after another
        begins = np.concatenate([[0], np.cumsum(runs)])
        ntubes = min(len(runs), 64)
        dt = 0.0
        n = 0
        for r in range(ntubes):
            sub = {k: np.asarray(v)[begins[r]:begins[r + 1]] for k, v in f.items()}
            sim = pyoracle.OracleSim(p, sub, kind=okind, flavor="fast", threads=threads)
            sim.initialize()
            for _ in range(warmup):
                sim.step()
            t0 = time.perf_counter()
            for _ in range(steps):
                sim.step()
            dt += time.perf_counter() - t0
            n += sim.n
            sim.close()
        sample = (f"{desc}: the first {ntubes} tubes ({n} particles) one after another, "
                  f"{warmup} untimed and {steps} timed steps each after an untimed initialize, "
                  f"{threads} OpenMP threads")
        return n * steps / dt, kind, sample, dt, steps, warmup
    sim = pyoracle.OracleSim(p, f, kind=okind, flavor="fast", threads=threads)
    t0 = time.perf_counter()
    sim.initialize()
    t_init = time.perf_counter() - t0
    t0 = time.perf_counter()
    done_w = 0
    for _ in range(warmup):
        sim.step()
        done_w += 1
        if budget_s is not None and time.perf_counter() - t0 > 0.5 * budget_s:
            break
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        sim.step()
        done += 1
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    n = sim.n
    sim.close()
    sample = (f"{desc}: {n} particles, Solver::initialize ({t_init:.1f} s, untimed), {done_w} untimed "
              f"and {done} timed Solver::integrate steps on {threads} OpenMP threads")
    return n * done / dt, kind, sample, dt, done, done_w


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # --warmup untimed and --steps timed steps of the reference, bounded to about a minute of
    # timed CPU work (the count actually run is reported)
    value, kind, sample, secs, steps, warm = cpu_reference_run(args.workload, max(1, args.steps), threads,
                                                              warmup=args.warmup, budget_s=60.0)
    _, _, desc, _ = workload(args.workload)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": secs / steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": desc},
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads,
                             "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---- GPU arm -----------------------------------------------------------------------------------
def adjoint_report():
    """The Gresho-Chan adjoint: 256 x 256 lattice (65,536 particles), ssph, cubic spline, 200
    steps at the fixed CFL dt of the initial state, a checkpoint every 20 steps, loss
    L = sum (rho_final - 1)^2, gradients in the initial velocities, the initial internal energy and
    avAlpha.  Reports the backward/forward wall-time ratio in both precisions, central finite
    differences of the FP64 forward pass over 20 steps, the FP32-pair gradient against FP64, and
    how far a 1e-12 velocity perturbation grows over the 200 steps."""
    from sphcode_gb300 import ics
    from sphcode_gb300.adjoint import cost_and_precision, finite_difference_check, perturbation_growth
    p, f = ics.gresho(256)
    steps, k, fd_steps = 200, 20, 20
    cost = cost_and_precision(p, f, steps, checkpoint_every=k)
    dt = cost["dt"]
    fd = finite_difference_check(p, f, fd_steps, dt, eps=1e-7)
    prec = cost_and_precision(p, f, fd_steps, dt=dt, checkpoint_every=k, reps=1)["fp32_vs_fp64"]
    growth = perturbation_growth(p, f, steps, dt)
    return {"workload": "gresho-chan 256x256 (65,536), ssph cubic, periodic, gamma 5/3, fixed dt "
                        "(initial CFL step), loss sum (rho_final - 1)^2",
            "steps": steps, "checkpoint_every": k, "dt": dt, "n_particles": int(f["mass"].size),
            "cost": {pr: cost[pr] for pr in ("fp32", "fp64")},
            "fd_check": {"steps": fd_steps, "eps": fd["eps"],
                         "directions": "dL/dv0 and dL/du0 along themselves, dL/davAlpha",
                         "rel_err": {"v0": fd["v"], "u0": fd["u"], "alpha": fd["alpha"]},
                         "adjoint": fd["adjoint"], "fd": fd["fd"]},
            "fp32_vs_fp64": {"steps": fd_steps, **prec},
            "fp32_vs_fp64_200_steps": cost["fp32_vs_fp64"],
            "perturbation_growth": {"size": 1e-12, "every": 20, "max_abs_drho": growth}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # about a second of timed KHI steps: the clock sampler (every 200 ms) sees several samples
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="khi")
    ap.add_argument("--ref-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--group-warps", type=int, default=0,
                    help="target-group size in warps (0 = the library's default)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the Gresho-Chan adjoint cost / finite-difference report")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-oracle", action="store_true",
                    help="skip the comparison with the reference's modules after initialize + 1 step")
    ap.add_argument("--no-workloads", action="store_true",
                    help="skip the FP32/FP64 summaries of the other workloads")
    ap.add_argument("--pass2-scale", type=int, default=0)
    ap.add_argument("--tile-pre", type=int, default=0)
    ap.add_argument("--tile-fluid", type=int, default=0)
    ap.add_argument("--profile-run", action="store_true",
                    help="initialize + --steps eager steps and exit (a short, fixed launch sequence "
                         "for ncu: no timing, graphs, CPU baseline or e2e)")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="Gresho 256x256: --steps steps forward and backward through the adjoint, then exit "
                         "(a short, fixed launch sequence for ncu)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference_arm(args)
        return
    if args.profile_adjoint:
        # a fixed, short launch sequence of the adjoint for ncu: the Gresho vortex (256 x 256),
        # initialize + --steps steps forward and their reversal, FP32-pair form
        import __graft_entry__ as g
        g.build()
        import torch
        from sphcode_gb300 import ics
        from sphcode_gb300.adjoint import SphRun
        p, f = ics.gresho(256)
        run = SphRun(p, f, args.steps, dt=5.915e-4, precision=args.precision, checkpoint_every=args.steps)
        rho = run.forward(torch.tensor(f["vel"], device="cuda"), torch.tensor(f["ene"], device="cuda"), p.av_alpha)
        run.backward(2 * (rho - 1))
        print(json.dumps({"profile_adjoint": "gresho 256x256", "steps": args.steps, "precision": args.precision}))
        run.close()
        return
    if args.profile_run:
        import __graft_entry__ as g
        g.build()
        from sphcode_gb300 import sphgpu
        p, f, desc, runs = workload(args.workload)
        with sphgpu.GpuSimulation(p, f, precision=args.precision, runs=runs) as sim:
            sim.set_tuning("graph", 0)
            if args.no_autotune:
                sim.set_tuning("autotune", 0)
            if args.group_warps:
                sim.set_tuning("group_warps", args.group_warps)
            if args.tile_pre:
                sim.set_tuning("tile_cap_pre", args.tile_pre)
            if args.tile_fluid:
                sim.set_tuning("tile_cap", args.tile_fluid)
            sim.initialize()
            sim.step(args.steps)
            print(json.dumps({"profile_run": desc, "n": sim.n, "steps": args.steps,
                              "precision": args.precision, "time": sim.scalar("time")}))
        return
    if args.warmup < 3:
        raise SystemExit("at least 3 warm-up steps")

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__ as g
    if rank == 0 or world == 1:
        g.build()
    if dist:
        dist.barrier()
    from sphcode_gb300 import sphgpu

    p, f, desc, runs = workload(args.workload)
    n = int(f["mass"].shape[0])
    D = p.dim

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- FP32-pair form: device-resident throughput --------------------------------------
    def make(prec):
        s_ = sphgpu.GpuSimulation(p, f, precision=prec, runs=runs)
        if args.group_warps:
            s_.set_tuning("group_warps", args.group_warps)
        if args.tile_pre:
            s_.set_tuning("tile_cap_pre", args.tile_pre)
        if args.tile_fluid:
            s_.set_tuning("tile_cap", args.tile_fluid)
        if args.pass2_scale:
            s_.set_tuning("pass2_scale", args.pass2_scale)
        return s_

    sim = make("fp32")
    sim.initialize()
    sim.step(args.warmup)
    launches_per_step = sim.get_tuning("graph_kernels")
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    clocks.mark()
    ms = sim.bench_steps(args.steps, flush_l2=True)
    barrier()
    clk = clocks.stop()
    ms, value = aggregate(ms, n, args.steps, dist, "cuda")

    # per-stage device times (eager launches, CUDA events between stages on the library's stream)
    sim.set_tuning("timing", 1)
    sim.step(1)
    stages = {k: 0.0 for k in ("tree", "pre", "fluid", "gravity", "integrate")}
    reps = 3
    for _ in range(reps):
        sim.step(1)
        for k, v in sim.stage_times().items():
            stages[k] += v / reps
    overflow = {"pre": sim.get_tuning("overflow_pre"), "fluid": sim.get_tuning("overflow_fluid")}
    # work counters of one more step (counted in a step of its own, outside every timed step)
    sim.set_tuning("count_work", 1)
    sim.pair_counters(reset=True)
    sim.step(1)
    counters = sim.pair_counters(reset=True)
    sim.set_tuning("count_work", 0)
    schedule = {"group_warps": sim.get_tuning("group_warps"), "tile_pre": sim.get_tuning("tile_cap_pre"),
                "tile_fluid": sim.get_tuning("tile_cap"), "pass2_scale": sim.get_tuning("pass2_scale"),
                "pair_sched": ["groups", "groups+tpp after pass 1", "groups+tpp after pass 2",
                               "thread-per-particle"][sim.get_tuning("pair_sched")],
                "group_rule": ["chunks", "key blocks"][sim.get_tuning("group_rule")],
                "autotuned": bool(sim.get_tuning("autotune")),
                "rejected_candidate_status_bits": sim.get_tuning("tune_rejects")}
    sim.set_tuning("timing", 0)
    pairs = sim.neighbor_counts(True).astype(np.int64) - 1   # r = 0 (self) is skipped
    mean_pairs = float(pairs.mean())
    newton_fail = sim.newton_failures()
    sim.close()

    # ---- FP64 plain form; both forms against the GPU FP64 form and the reference -------------
    fp64 = None
    errs, errs_oracle, errs64_oracle = {}, None, None
    fields_cmp = ("dens", "sml", "pres", "acc", "dene", "pos", "vel", "ene")

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))

    if not args.no_fp64:
        s64 = make("fp64")
        s32 = make("fp32")
        s64.initialize()
        s32.initialize()
        s64.step(1)
        s32.step(1)
        got32 = {k: s32.get(k) for k in fields_cmp}
        got64 = {k: s64.get(k) for k in fields_cmp}
        errs = {k: rel(got32[k], got64[k]) for k in fields_cmp}
        s32.close()
        if rank == 0 and world == 1 and not args.no_oracle:
            ref = oracle_step(p, f)
            errs_oracle = {k: rel(got32[k], ref[k]) for k in fields_cmp}
            errs64_oracle = {k: rel(got64[k], ref[k]) for k in fields_cmp}
        s64.step(args.warmup - 1)
        k64 = max(3, args.steps // 4)
        barrier()
        ms64 = max_over_ranks(s64.bench_steps(k64, flush_l2=True))
        fp64 = {"value": world * n * k64 / (ms64 * 1e-3), "steps": k64, "ms_per_step": ms64 / k64}
        s64.close()

    # ---- end to end through the reference-facing AoS boundary, host buffers ------------------
    e2e = None
    if not args.no_e2e:
        dt = aos_dtype(D)
        holder, raw = pinned_array(n * dt.itemsize)
        aos = raw.view(dt)
        aos[:] = 0
        aos["pos"] = f["pos"].reshape(n, D)
        aos["vel"] = f["vel"].reshape(n, D)
        aos["mass"] = f["mass"]
        aos["dens"] = f["dens"]
        aos["pres"] = f["pres"]
        aos["ene"] = f["ene"]
        aos["id"] = np.arange(n)
        lay = aos_layout(dt)
        import ctypes
        e2e_sim = make("fp32")
        # the Module pattern (upload, calculate, download) leaves the record members outside the
        # layout untouched on the host between an upload and the next download
        e2e_sim.set_tuning("aos_reuse", 1)
        e2e_sim.initialize()
        e2e_sim.lib.sphgpu_download_aos(e2e_sim._h, ctypes.c_void_p(raw.ctypes.data), ctypes.byref(lay))
        e2e_sim.step(args.warmup)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rc = e2e_sim.lib.sphgpu_upload_aos(e2e_sim._h, ctypes.c_void_p(raw.ctypes.data), ctypes.byref(lay))
            rc |= e2e_sim.lib.sphgpu_step(e2e_sim._h, 1)
            rc |= e2e_sim.lib.sphgpu_download_aos(e2e_sim._h, ctypes.c_void_p(raw.ctypes.data), ctypes.byref(lay))
            if rc:
                raise RuntimeError(e2e_sim.lib.sphgpu_last_error(e2e_sim._h))
        barrier()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        e2e_sim.close()
        e2e = {"value": world * n * args.steps / e2e_s, "unit": "particle-steps/s",
               "h2d_bytes_per_step": n * dt.itemsize, "d2h_bytes_per_step": n * dt.itemsize,
               "path": "sphgpu_upload_aos + sphgpu_step(1) + sphgpu_download_aos, pinned "
                       "SPHParticle-layout buffer, record reuse on"}

    # ---- rooflines: every pair stage, the dominant one as `roofline` -----------------------------
    fp32_peak, fp64_peak = sphgpu.measure_peaks()
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s"

    def line_for(kernel, flops, ms, nbytes, extra):
        ach = flops / (ms * 1e-3) / 1e12 if ms > 0 else 0.0
        gbs = nbytes / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        out = {"kernel": kernel, "bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
               "frac": ach / fp32_peak if fp32_peak > 0 else None, "traffic": None,
               "algorithmic_flops_per_launch": flops, "launch_ms": ms,
               "peak_source": "sphgpu_measure_peaks FP32 FMA loop on this GPU (of measured)",
               "hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                       "algorithmic_bytes_per_launch": nbytes, "peak_source": hbm_src}}
        out.update(extra)
        return out

    flops_pair = FLUID_FLOPS_PER_PAIR.get((p.sph_type, D), 120)
    fnew = PRE_NEWTON_FLOPS_PER_PAIR[D]
    fden = PRE_DENS_FLOPS_PER_PAIR.get((p.sph_type, D), 90)
    pre_flops = counters["pre_iter_pairs"] * fnew + counters["pre_pairs"] * fden
    tgt = max(counters["pre_targets"], 1)
    rooflines = {
        "pre": line_for("pre_kernel (PreInteraction, FP32 pairs; all passes + mirror)", pre_flops, stages["pre"],
                        pre_bytes_per_particle(D) * n,
                        {"newton_iterations_per_particle": counters["pre_iters"] / tgt,
                         "neighbours_per_particle": counters["pre_pairs"] / tgt,
                         "candidates_per_particle": counters["pre_candidates"] / tgt,
                         "staged_sources_tested_per_particle": counters["pre_tests"] / tgt,
                         "flops_per_pair": {"newton": fnew, "density": fden},
                         "work_source": "device counters of one step (sphgpu_pair_counters)"}),
        "fluid": line_for("fluid_kernel (FluidForce, FP32 pairs; all passes + mirror)", mean_pairs * n * flops_pair,
                          stages["fluid"], fluid_bytes_per_particle(D) * n,
                          {"pairs_per_particle": mean_pairs, "flops_per_pair": flops_pair,
                           "staged_sources_tested_per_particle": counters["fluid_tests"] / max(n, 1)}),
    }
    if p.use_gravity and counters.get("grav_nodes", 0) + counters.get("grav_pairs", 0) > 0:
        gflops = counters["grav_nodes"] * GRAV_FLOPS_NODE + counters["grav_pairs"] * GRAV_FLOPS_LEAF
        rooflines["gravity"] = line_for("gravity_kernel (Barnes-Hut walk, FP32 terms)", gflops, stages["gravity"],
                                        grav_bytes_per_particle(D) * n,
                                        {"monopoles_per_particle": counters["grav_nodes"] / max(n, 1),
                                         "leaf_pairs_per_particle": counters["grav_pairs"] / max(n, 1),
                                         "flops_per_term": {"monopole": GRAV_FLOPS_NODE, "leaf_pair": GRAV_FLOPS_LEAF},
                                         "work_source": "device counters of one step (sphgpu_pair_counters)"})
    # the dominant stage among those with a roofline entry
    dom = max((k for k in ("pre", "fluid", "gravity") if k in rooflines), key=lambda k: stages[k])
    roofline = dict(rooflines[dom])
    roofline["dominant_stage"] = dom
    if args.workload == "khi":
        # DRAM bytes of one launch of the dominant pair kernel from the committed ncu capture
        import re
        try:
            prof = open(os.path.join(ROOT, "profiles", "pair_kernels_khi_786k_fp32.md")).read()
            m = re.search(r"traffic_bytes_per_launch %s_kernel: (\d+)" % dom, prof)
            if m:
                roofline["traffic"] = int(m.group(1))
                roofline["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum of pass 1, " \
                                             "profiles/pair_kernels_khi_786k_fp32.md"
        except OSError:
            pass

    # ---- CPU baseline (rank 0, N = 1) -------------------------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, kind, sample, _, _, _ = cpu_reference_run(args.workload, args.ref_steps, threads)
        cpu = {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": kind, "sample": sample}

    adjoint = None
    if rank == 0 and world == 1 and not args.no_adjoint:
        adjoint = adjoint_report()

    others = {}
    if rank == 0 and world == 1 and not args.no_workloads:
        for name in ("evrard", "ensemble", "gresho"):
            if name != args.workload:
                others[name] = workload_summary(name, make_sim=None)

    if rank == 0:
        def r3(x):
            return None if x is None else float(f"{x:.3g}")
        summary = {
            "fp32_value": r3(value), "fp64_value": r3(fp64["value"]) if fp64 else None,
            "fp32_over_fp64": r3(value / fp64["value"]) if fp64 else None,
            "fp32_rel_err_vs_fp64": {k: r3(v) for k, v in errs.items()},
            "fp32_rel_err_vs_oracle": {k: r3(v) for k, v in errs_oracle.items()} if errs_oracle else None,
            "fp64_rel_err_vs_oracle": {k: r3(v) for k, v in errs64_oracle.items()} if errs64_oracle else None,
            "oracle": "reference modules, strict FP64, initialize + 1 step" if errs_oracle else None,
            "roofline": {"kernel": dom, "tflops": r3(roofline["achieved"]), "frac": r3(roofline["frac"])},
            "workloads": {k: {"fp32": r3(v["fp32"]), "fp64": r3(v["fp64"]), "ratio": r3(v["ratio"])}
                          for k, v in others.items()},
            "adjoint": ({"bwd_over_fwd_fp32": r3(adjoint["cost"]["fp32"]["backward_over_forward"]),
                         "bwd_over_fwd_fp64": r3(adjoint["cost"]["fp64"]["backward_over_forward"]),
                         "fd_rel_err_20_steps": {k: r3(v) for k, v in adjoint["fd_check"]["rel_err"].items()},
                         "fp32_vs_fp64_200_steps": {k: r3(v) for k, v in adjoint["fp32_vs_fp64_200_steps"].items()},
                         "note": "the FP32-pair gradient over 200 steps is not usable (see fp32_vs_fp64_200_steps); "
                                 "the cost claim holds for the FP64 gradient and for FP32 over <= 20 steps"}
                        if adjoint else None),
        }
        line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": desc, "n_particles": n, "dim": D, "sph_type": p.sph_type,
                           "kernel": p.kernel, "neighbor_number": p.neighbor_number,
                           "form": "fp32_pair (FP32 pair sums, Kahan totals, FP64 state)",
                           "l2": "2 x L2 buffer overwritten between timed steps",
                           "parallelism": f"replicas{world}"},
                "adjoint": adjoint, "workloads": others,
                "stage_ms": stages, "overflow_groups": overflow, "newton_failures": newton_fail,
                "schedule": schedule, "work_counters": counters, "rooflines": rooflines,
                "peaks": {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak},
                "fp64_form": fp64, "fp32_over_fp64": (value / fp64["value"]) if fp64 else None,
                "fp32_rel_err_vs_fp64_after_1_step": errs,
                "fp32_rel_err_vs_oracle_after_1_step": errs_oracle,
                "fp64_rel_err_vs_oracle_after_1_step": errs64_oracle,
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": launches_per_step * args.steps,
                "summary": summary}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def oracle_step(p, f):
    """The reference's own modules (strict FP64 flavour; the C restatement where they are not
    built) after initialize + 1 step, on every host core: the fields the bench compares."""
    from oracle import pyoracle
    kind = "ref" if pyoracle.reference_available("strict") else "port"
    ref = pyoracle.OracleSim(p, f, kind=kind, flavor="strict", threads=os.cpu_count())
    ref.initialize()
    ref.step()
    out = {k: ref.get(k) for k in ("dens", "sml", "pres", "acc", "dene", "pos", "vel", "ene")}
    ref.close()
    return out


def workload_summary(name, make_sim=None, steps=20, steps64=4):
    """FP32-pair and FP64 particle-steps/s of another workload (initialize with the tuner, 3
    warm-up steps, then timed steps with the L2 flushed between them)."""
    from sphcode_gb300 import sphgpu
    p, f, desc, runs = workload(name)
    n = int(f["mass"].shape[0])
    out = {"workload": desc, "n_particles": n}
    for prec, k in (("fp32", steps), ("fp64", steps64)):
        with sphgpu.GpuSimulation(p, f, precision=prec, runs=runs) as sim:
            sim.initialize()
            sim.step(3)
            ms = sim.bench_steps(k, flush_l2=True)
            out[prec] = n * k / (ms * 1e-3)
            out[prec + "_ms_per_step"] = ms / k
            if prec == "fp32":
                sim.set_tuning("timing", 1)
                sim.step(1)
                out["fp32_stage_ms"] = {kk: round(v, 4) for kk, v in sim.stage_times().items()}
                out["fp32_overflow_groups"] = {"pre": sim.get_tuning("overflow_pre"),
                                               "fluid": sim.get_tuning("overflow_fluid")}
                sim.set_tuning("timing", 0)
                out["fp32_schedule"] = {"group_warps": sim.get_tuning("group_warps"),
                                        "tile_pre": sim.get_tuning("tile_cap_pre"),
                                        "tile_fluid": sim.get_tuning("tile_cap"),
                                        "pair_sched": sim.get_tuning("pair_sched"),
                                        "group_rule": sim.get_tuning("group_rule")}
    out["ratio"] = out["fp32"] / out["fp64"]
    return out


if __name__ == "__main__":
    main()
