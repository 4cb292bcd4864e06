"""Synthetic initial conditions for the benchmarked workloads.

Each generator returns ``(params, fields)`` where ``fields`` maps field names to float64 numpy
arrays in particle order (vector fields shaped ``(N, DIM)``).  The shapes, sizes and value
distributions are those of the workloads the reference is measured on; the reference's own
sample generators (src/sample/*.cpp) use different lattices and are noted per function.
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np

from .params import SPHParameters

Fields = Dict[str, np.ndarray]


def sod(n_left: int = 800, n_right: int = 100) -> Tuple[SPHParameters, Fields]:
    """1D Sod shock tube, plain ssph with the cubic spline: x in [-0.5, 0.5], n_left equally
    spaced particles on [-0.5, 0) with rho = 1, p = 1 and n_right on [0, 0.5] with rho = 0.125,
    p = 0.1; equal mass; v = 0; gamma = 1.4; neighborNumber 4; avAlpha 1; endTime 0.2;
    not periodic.  (src/sample/shock_tube.cpp uses 400/100 particles with other states.)"""
    p = SPHParameters(dim=1, sph_type="ssph", kernel="cubic_spline", gamma=1.4, neighbor_number=4,
                      av_alpha=1.0, end_time=0.2, periodic=False)
    dxl = 0.5 / n_left
    dxr = 0.5 / n_right
    xl = -0.5 + (np.arange(n_left) + 0.5) * dxl
    xr = (np.arange(n_right) + 0.5) * dxr
    x = np.concatenate([xl, xr])
    rho = np.concatenate([np.full(n_left, 1.0), np.full(n_right, 0.125)])
    pres = np.concatenate([np.full(n_left, 1.0), np.full(n_right, 0.1)])
    mass = np.full(x.size, 1.0 * dxl)
    ene = pres / ((p.gamma - 1.0) * rho)
    f = dict(pos=x.reshape(-1, 1), vel=np.zeros((x.size, 1)), mass=mass, dens=rho, pres=pres, ene=ene)
    return p, f


def khi(n_in: int = 1024, n_out: int = 724) -> Tuple[SPHParameters, Fields]:
    """2D Kelvin-Helmholtz instability, disph + Wendland C4 + artificial conductivity, periodic
    unit box, gamma = 5/3, p = 2.5.  The strip |y - 0.5| < 0.25 is a square lattice of spacing
    1/n_in with rho = 2, vx = -0.5; outside, a square lattice of spacing 1/n_out with rho = 1,
    vx = +0.5; all particles have the mass 2/n_in^2.  vy = 0.1 sin(4 pi x) [exp(-(y-0.25)^2/0.005)
    + exp(-(y-0.75)^2/0.005)] (two Gaussians, as src/sample/khi.cpp:33-36 adds them).
    neighborNumber 64, endTime 2, leafParticleNumber 16, Balsara switch and time-dependent AV as
    in sample/khi/khi.json.  Default sizes give 786,376 particles."""
    p = SPHParameters(dim=2, sph_type="disph", kernel="wendland", gamma=5.0 / 3.0,
                      neighbor_number=64, end_time=2.0, leaf_num=16, use_balsara=True,
                      use_tdav=True, use_ac=True, alpha_ac=1.0, periodic=True,
                      range_min=[0.0, 0.0, 0.0], range_max=[1.0, 1.0, 0.0])
    yi = (np.arange(n_in) + 0.5) / n_in
    yi = yi[np.abs(yi - 0.5) < 0.25]
    xi = (np.arange(n_in) + 0.5) / n_in
    yo = (np.arange(n_out) + 0.5) / n_out
    yo = yo[np.abs(yo - 0.5) >= 0.25]
    xo = (np.arange(n_out) + 0.5) / n_out
    Xi, Yi = np.meshgrid(xi, yi)
    Xo, Yo = np.meshgrid(xo, yo)
    x = np.concatenate([Xo.ravel(), Xi.ravel()])
    y = np.concatenate([Yo.ravel(), Yi.ravel()])
    inner = np.concatenate([np.zeros(Xo.size, bool), np.ones(Xi.size, bool)])
    # order particles row by row (lower outer rows, strip, upper outer rows) like a lattice scan
    order = np.lexsort((x, y))
    x, y, inner = x[order], y[order], inner[order]
    n = x.size
    rho = np.where(inner, 2.0, 1.0)
    pres = np.full(n, 2.5)
    vx = np.where(inner, -0.5, 0.5)
    vy = 0.1 * np.sin(4.0 * math.pi * x) * (np.exp(-(y - 0.25) ** 2 / 0.005) + np.exp(-(y - 0.75) ** 2 / 0.005))
    mass = np.full(n, 2.0 / (n_in * n_in))
    ene = pres / ((p.gamma - 1.0) * rho)
    f = dict(pos=np.stack([x, y], 1), vel=np.stack([vx, vy], 1), mass=mass, dens=rho, pres=pres, ene=ene)
    return p, f


def evrard(n: int = 1 << 20, seed: int = 20261203) -> Tuple[SPHParameters, Fields]:
    """3D Evrard collapse with self-gravity, disph + Wendland C4 + Balsara + time-dependent AV,
    gamma = 5/3, G = 1, theta = 0.5: n equal-mass particles in a sphere of radius 1 and mass 1
    with rho ~ 1/r (radius r = sqrt(s), s ~ U(0,1) from the seed, isotropic directions), initial
    density 1/(2 pi r) for the smoothing-length guess (src/sample/evrard.cpp:58), u = 0.05, v = 0,
    neighborNumber 50, leafParticleNumber 32 (sample/evrard/evrard.json), endTime 3.
    (src/sample/evrard.cpp stretches a cubic lattice instead of sampling.)"""
    p = SPHParameters(dim=3, sph_type="disph", kernel="wendland", gamma=5.0 / 3.0,
                      neighbor_number=50, end_time=3.0, leaf_num=32, use_balsara=True,
                      use_tdav=True, use_gravity=True, g_constant=1.0, theta=0.5, periodic=False)
    rng = np.random.default_rng(seed)
    s = rng.random(n)
    r = np.sqrt(s)
    cth = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * math.pi, n)
    sth = np.sqrt(1.0 - cth * cth)
    pos = np.stack([r * sth * np.cos(phi), r * sth * np.sin(phi), r * cth], 1)
    rr = np.sqrt((pos * pos).sum(1))
    dens = 1.0 / (2.0 * math.pi * rr)
    u = 0.05 * p.g_constant
    f = dict(pos=pos, vel=np.zeros((n, 3)), mass=np.full(n, 1.0 / n), dens=dens,
             pres=(p.gamma - 1.0) * dens * u, ene=np.full(n, u))
    return p, f


def gresho(n_side: int = 256) -> Tuple[SPHParameters, Fields]:
    """2D Gresho-Chan vortex, ssph + cubic spline, periodic [-0.5, 0.5]^2, n_side^2 lattice,
    rho = 1, gamma = 5/3; v_phi = 5r (r < 0.2), 2 - 5r (0.2 <= r < 0.4), 0 beyond;
    p = 5 + 12.5 r^2, 9 + 12.5 r^2 - 20 r + 4 ln(5r), 3 + 4 ln 2 in the same bands
    (src/sample/gresho_chan_vortex.cpp:12-32,40-70); neighborNumber 32."""
    p = SPHParameters(dim=2, sph_type="ssph", kernel="cubic_spline", gamma=5.0 / 3.0,
                      neighbor_number=32, end_time=1.0, leaf_num=32, use_balsara=True,
                      periodic=True, range_min=[-0.5, -0.5, 0.0], range_max=[0.5, 0.5, 0.0])
    dx = 1.0 / n_side
    c = -0.5 + (np.arange(n_side) + 0.5) * dx
    X, Y = np.meshgrid(c, c)
    x, y = X.ravel(), Y.ravel()
    r = np.sqrt(x * x + y * y)
    vphi = np.where(r < 0.2, 5.0 * r, np.where(r < 0.4, 2.0 - 5.0 * r, 0.0))
    with np.errstate(divide="ignore"):
        pres = np.where(r < 0.2, 5.0 + 12.5 * r * r,
                        np.where(r < 0.4, 9.0 + 12.5 * r * r - 20.0 * r + 4.0 * np.log(np.maximum(5.0 * r, 1e-300)),
                                 3.0 + 4.0 * math.log(2.0)))
    vel = np.stack([-y / r * vphi, x / r * vphi], 1)
    n = x.size
    rho = np.ones(n)
    ene = pres / ((p.gamma - 1.0) * rho)
    f = dict(pos=np.stack([x, y], 1), vel=vel, mass=np.full(n, 1.0 / n), dens=rho, pres=pres, ene=ene)
    return p, f


def shock_tube_gsph(n_left: int, n_right: int, rho_l: float, rho_r: float, p_l: float, p_r: float,
                    neighbor_number: int = 4) -> Tuple[SPHParameters, Fields]:
    """One 1D tube of the gsph ensemble: x in [-0.5, 0.5], interface at 0, equal mass within the
    tube, particles split n_left / n_right, states (rho, p) left and right, gamma = 1.4, 2nd-order
    gsph with the cubic spline, not periodic."""
    p = SPHParameters(dim=1, sph_type="gsph", kernel="cubic_spline", gamma=1.4,
                      neighbor_number=neighbor_number, gsph_2nd_order=True, periodic=False)
    xl = -0.5 + (np.arange(n_left) + 0.5) * (0.5 / n_left)
    xr = (np.arange(n_right) + 0.5) * (0.5 / n_right)
    x = np.concatenate([xl, xr])
    rho = np.concatenate([np.full(n_left, rho_l), np.full(n_right, rho_r)])
    pres = np.concatenate([np.full(n_left, p_l), np.full(n_right, p_r)])
    mass = np.full(x.size, rho_l * 0.5 / n_left)
    f = dict(pos=x.reshape(-1, 1), vel=np.zeros((x.size, 1)), mass=mass, dens=rho, pres=pres,
             ene=pres / ((p.gamma - 1.0) * rho))
    return p, f


def ensemble_tubes(n_runs: int = 4096, n_min: int = 200, n_max: int = 5000, seed: int = 20261203):
    """The gsph ensemble: n_runs independent tubes with particle counts ~ U{n_min..n_max},
    rho_L, rho_R, p_L, p_R log-uniform in [0.1, 1] from the seed, particle split
    n_L / n_R = rho_L / rho_R (equal mass within a tube).  Returns a list of per-tube dicts."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(n_min, n_max + 1, n_runs)
    states = np.exp(rng.uniform(math.log(0.1), math.log(1.0), (n_runs, 4)))
    tubes = []
    for k in range(n_runs):
        rl, rr, pl, pr = states[k]
        nl = int(round(counts[k] * rl / (rl + rr)))
        nl = min(max(nl, 1), counts[k] - 1)
        tubes.append(dict(n_left=nl, n_right=int(counts[k] - nl), rho_l=rl, rho_r=rr, p_l=pl, p_r=pr))
    return tubes


def ensemble(n_runs: int = 4096, n_min: int = 200, n_max: int = 5000, seed: int = 20261203):
    """The gsph ensemble as one batch: ``(params, fields, run_sizes)`` with the tubes of
    :func:`ensemble_tubes` stored back to back (each tube keeps its own coordinates in
    [-0.5, 0.5]; runs never interact)."""
    tubes = ensemble_tubes(n_runs, n_min, n_max, seed)
    parts = [shock_tube_gsph(t["n_left"], t["n_right"], t["rho_l"], t["rho_r"], t["p_l"], t["p_r"])
             for t in tubes]
    p = parts[0][0]
    names = parts[0][1].keys()
    fields = {k: np.concatenate([f[k] for _, f in parts]) for k in names}
    sizes = [int(f["mass"].shape[0]) for _, f in parts]
    return p, fields, sizes


# ---- the reference's sample initial conditions (src/sample/*.cpp) ------------------------------
# Restated operation for operation in IEEE double (Python floats and the C library's scalar
# sqrt/pow/sin/exp/log, as the reference calls them), including the sequential coordinate
# accumulation (x += dx), so that positions and states are bit-identical to the reference's.
# Each returns the particle fields in the reference's particle order (id == index).  The sample
# sizes are small (N from the sample's JSON file), so the generators run on the host.

SAMPLE_DIM = {"shock_tube": 1, "gresho_chan_vortex": 2, "pairing_instability": 2, "hydrostatic": 2,
              "khi": 2, "evrard": 3}


def _fields_from(pos, vel, mass, dens, pres, ene, dim):
    n = len(mass)
    return dict(pos=np.asarray(pos, dtype=np.float64).reshape(n, dim),
                vel=np.asarray(vel, dtype=np.float64).reshape(n, dim),
                mass=np.asarray(mass, dtype=np.float64), dens=np.asarray(dens, dtype=np.float64),
                pres=np.asarray(pres, dtype=np.float64), ene=np.asarray(ene, dtype=np.float64))


def sample_shock_tube(N: int, gamma: float) -> Fields:
    """Solver::make_shock_tube (src/sample/shock_tube.cpp:12-50): 10 N particles, left state
    rho 1, p 1 at spacing 0.5/N/4 from x = -0.5, right state rho 0.25, p 0.1795 at spacing 0.5/N
    after x passes 0.5."""
    dx_r = 0.5 / N
    dx_l = dx_r * 0.25
    num = N * 10
    x, dx, dens, pres = -0.5 + dx_l * 0.5, dx_l, 1.0, 1.0
    mass = 0.5 / N * 0.25
    left = True
    P, D, PR = [], [], []
    for _ in range(num):
        P.append(x)
        D.append(dens)
        PR.append(pres)
        x += dx
        if x > 0.5 and left:
            x = 0.5 + dx_r * 0.5
            dx = dx_r
            dens = 0.25
            pres = 0.1795
            left = False
    ene = [pr / ((gamma - 1.0) * d) for pr, d in zip(PR, D)]
    return _fields_from(P, [0.0] * num, [mass] * num, D, PR, ene, 1)


def sample_khi(N: int, gamma: float) -> Fields:
    """Solver::make_khi (src/sample/khi.cpp:12-80): 3 N^2 / 4 particles; outer layers (region 1:
    rho 1, vx -0.5) on rows of spacing 1/N with every other column, staggered by row; the strip
    0.25 < y < 0.75 (region 2: rho 2, vx +0.5) on the full 1/N lattice; p = 2.5; vy of two
    Gaussians of width 0.05 around y = 0.25 and 0.75."""
    num = N * N * 3 // 4
    dx = 1.0 / N
    mass = 1.5 / num
    sigma2_inv = 2 / (0.05 * 0.05)

    def vy(x, y):
        return 0.1 * math.sin(4.0 * math.pi * x) * (math.exp(-((y - 0.25) * (y - 0.25)) * 0.5 * sigma2_inv)
                                                  + math.exp(-((y - 0.75) * (y - 0.75)) * 0.5 * sigma2_inv))

    x = dx * 0.5
    y = dx * 0.5
    region, odd = 1, True
    P, V, D = [], [], []
    for _ in range(num):
        P += [x, y]
        V += [-0.5 if region == 1 else 0.5, vy(x, y)]
        D.append(float(region))
        x += 2.0 * dx if region == 1 else dx
        if x > 1.0:
            y += dx
            region = 2 if (y > 0.25 and y < 0.75) else 1
            if region == 1:
                if odd:
                    odd = False
                    x = dx * 1.5
                else:
                    odd = True
                    x = dx * 0.5
            else:
                x = dx * 0.5
    pres = [2.5] * num
    ene = [2.5 / ((gamma - 1.0) * d) for d in D]
    return _fields_from(P, V, [mass] * num, D, pres, ene, 2)


def sample_evrard(N: int, gamma: float, G: float) -> Fields:
    """Solver::make_evrard (src/sample/evrard.cpp:12-58): the cells of an N^3 lattice on
    [-1, 1]^3 within the unit sphere, each radius r0 stretched to r0^1.5 (rho ~ 1/r), total mass
    1, u = 0.05 G, initial density 1 / (2 pi r)."""
    dx = 2.0 / N
    P = []
    for i in range(N):
        for j in range(N):
            for k in range(N):
                r = [(i + 0.5) * dx - 1.0, (j + 0.5) * dx - 1.0, (k + 0.5) * dx - 1.0]
                r0 = math.sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2])
                if r0 > 1.0:
                    continue
                if r0 > 0.0:
                    s = math.pow(r0, 1.5) / r0
                    r = [r[0] * s, r[1] * s, r[2] * s]
                P.append(r)
    num = len(P)
    mass = 1.0 / num
    u = 0.05 * G
    D = [1.0 / (2.0 * math.pi * math.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2])) for q in P]
    pres = [(gamma - 1.0) * d * u for d in D]
    return _fields_from(P, [0.0] * (3 * num), [mass] * num, D, pres, [u] * num, 3)


def _vortex_velocity(r):
    if r < 0.2:
        return 5.0 * r
    if r < 0.4:
        return 2.0 - 5.0 * r
    return 0.0


def _vortex_pressure(r):
    if r < 0.2:
        return 5.0 + 12.5 * r * r
    if r < 0.4:
        return 9.0 + 12.5 * r * r - 20.0 * r + 4.0 * math.log(5.0 * r)
    return 3.0 + 4.0 * math.log(2.0)


def sample_gresho_chan_vortex(N: int, gamma: float) -> Fields:
    """Solver::make_gresho_chan_vortex (src/sample/gresho_chan_vortex.cpp:12-74): N^2 lattice on
    [-0.5, 0.5]^2, rho 1, the vortex velocity and pressure of Gresho & Chan (1990)."""
    dx = 1.0 / N
    num = N * N
    x = -0.5 + dx * 0.5
    y = -0.5 + dx * 0.5
    mass = 1.0 / num
    P, V, PR = [], [], []
    for _ in range(num):
        P += [x, y]
        r = math.sqrt(x * x + y * y)
        vel = _vortex_velocity(r)
        dx_, dy_ = -y / r, x / r
        V += [dx_ * vel, dy_ * vel]
        PR.append(_vortex_pressure(r))
        x += dx
        if x > 0.5:
            x = -0.5 + dx * 0.5
            y += dx
    ene = [pr / ((gamma - 1.0) * 1.0) for pr in PR]
    return _fields_from(P, V, [mass] * num, [1.0] * num, PR, ene, 2)


def sample_hydrostatic(N: int, gamma: float) -> Fields:
    """Solver::make_hydrostatic (src/sample/hydrostatic.cpp:12-74): a dense square (rho 4) of
    spacing 0.5/N in |x|, |y| < 0.25 and an ambient medium (rho 1) of twice the spacing around
    it, equal masses 1/N^2, p = 2.5 everywhere (Saitoh & Makino 2013)."""
    dx1 = 0.5 / N
    dx2 = dx1 * 2.0
    mass = 1.0 / (N * N)
    P, D = [], []
    x = -0.25 + dx1 * 0.5
    y = -0.25 + dx1 * 0.5
    while y < 0.25:
        P += [x, y]
        D.append(4.0)
        x += dx1
        if x > 0.25:
            x = -0.25 + dx1 * 0.5
            y += dx1
    x = -0.5 + dx2 * 0.5
    y = -0.5 + dx2 * 0.5
    while y < 0.5:
        P += [x, y]
        D.append(1.0)
        while True:
            x += dx2
            if x > 0.5:
                x = -0.5 + dx2 * 0.5
                y += dx2
            if not (x > -0.25 and x < 0.25 and y > -0.25 and y < 0.25):
                break
    num = len(D)
    ene = [2.5 / ((gamma - 1.0) * d) for d in D]
    return _fields_from(P, [0.0] * (2 * num), [mass] * num, D, [2.5] * num, ene, 2)


class _MT19937:
    """The 32-bit Mersenne Twister of Matsumoto & Nishimura (1998) with the standard integer
    seeding (std::mt19937(seed))."""

    def __init__(self, seed: int):
        self.mt = [0] * 624
        self.mt[0] = seed & 0xFFFFFFFF
        for i in range(1, 624):
            prev = self.mt[i - 1]
            self.mt[i] = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
        self.idx = 624

    def _twist(self):
        mt = self.mt
        for i in range(624):
            y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
            v = mt[(i + 397) % 624] ^ (y >> 1)
            if y & 1:
                v ^= 0x9908B0DF
            mt[i] = v
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= 624:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF


def _uniform_real(eng: _MT19937, a: float, b: float) -> float:
    """std::uniform_real_distribution<double>(a, b) over a 32-bit engine as the GNU C++ library
    forms it: a canonical value from two draws, (x0 + x1 2^32) / 2^64 (clamped below 1), then
    u (b - a) + a."""
    x0 = eng()
    x1 = eng()
    u = (float(x0) + float(x1) * 4294967296.0) / 18446744073709551616.0
    if u >= 1.0:
        u = math.nextafter(1.0, 0.0)
    return u * (b - a) + a


def sample_pairing_instability(N: int, gamma: float) -> Fields:
    """Solver::make_pairing_instability (src/sample/pairing_instability.cpp:12-53): N^2 lattice on
    [-0.5, 0.5]^2 displaced by uniform offsets in +-0.05 dx from std::mt19937(1), rho 1, p 1."""
    dx = 1.0 / N
    num = N * N
    x = -0.5 + dx * 0.5
    y = -0.5 + dx * 0.5
    mass = 1.0 / num
    eng = _MT19937(1)
    lo, hi = -dx * 0.05, dx * 0.05
    P = []
    for _ in range(num):
        px = x + _uniform_real(eng, lo, hi)
        py = y + _uniform_real(eng, lo, hi)
        P += [px, py]
        x += dx
        if x > 0.5:
            x = -0.5 + dx * 0.5
            y += dx
    ene = [1.0 / ((gamma - 1.0) * 1.0)] * num
    return _fields_from(P, [0.0] * (2 * num), [mass] * num, [1.0] * num, [1.0] * num, ene, 2)


def reference_sample(name: str, sample_root: str) -> Tuple[SPHParameters, Fields]:
    """A sample as the reference's `sph <sample>` runs it: the parameters of
    sample/<name>/<name>.json under `sample_root` (read like Solver::read_parameterfile,
    src/solver.cpp:163-191) and the initial condition of src/sample/<name>.cpp."""
    dim = SAMPLE_DIM[name]
    p = SPHParameters.from_json(name, dim, sample_root=sample_root)
    N, g = p.sample_n, p.gamma
    if name == "shock_tube":
        f = sample_shock_tube(N, g)
    elif name == "khi":
        f = sample_khi(N, g)
    elif name == "evrard":
        f = sample_evrard(N, g, p.g_constant)
    elif name == "gresho_chan_vortex":
        f = sample_gresho_chan_vortex(N, g)
    elif name == "hydrostatic":
        f = sample_hydrostatic(N, g)
    else:
        f = sample_pairing_instability(N, g)
    return p, f
