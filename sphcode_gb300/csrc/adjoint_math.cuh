// Reverse-mode (adjoint) algebra of one standard-SPH step, usable on host and device.
//
// Forward quantities at PreInteraction / FluidForce time (src/pre_interaction.cpp:39-169,
// src/fluid_force.cpp:26-106): positions x, velocities v, internal energy u, sound speed c,
// smoothing length h (the Newton root of rho(h) h^D = m N / A), density rho = sum m W(r, h),
// pressure P = (gamma - 1) rho u, grad-h term g = 1 / (1 + h rho_h / (D rho)) with
// rho_h = sum m dW/dh, Balsara switch B = |div v| / (|div v| + |rot v| + 1e-4 c / h) and the
// pair accelerations / energy rates with the Monaghan viscosity.  Neighbour sets and the
// viscosity branch (v_ij . r_ij < 0) are those of the forward pass.
//
// Three pieces:
//   fluid_pair_vjp     : vector-Jacobian product of one pair term of a_t and du_t;
//   pre_local_backward : per particle, from the adjoints of rho, P, g, h, c, B to the weights
//                        of its density-type pair sums, with the implicit h (F(h, x) = 0:
//                        dh/dx = -F_x / F_h) folded into the density weight;
//   pre_pair_gather    : the pair terms of those sums' position / velocity derivatives.
#pragma once

#include "kderiv.cuh"

namespace sphadj {

template <typename T>
struct FluidSide {
    T v[3];
    T rho, P, g, B, c, h, m;
    T u;                   // internal energy (pressure-energy form)
    T abar[3], dubar;      // adjoints of this particle's a and du
};

template <typename T>
struct SideAdj {
    T x[3], v[3];
    T rho, P, g, h, c, B;
    T u;                   // direct dependence on u (pressure-energy form)
    SPH_HD void zero()
    {
        for (int k = 0; k < 3; ++k) { x[k] = T(0); v[k] = T(0); }
        rho = P = g = h = c = B = u = T(0);
    }
};

// a_t += m_s r_ts Q, du_t += m_s (v_ts . r_ts) S with
//   Q = -(F_t A_t + F_s A_s + Pi (F_t + F_s) / 2),  S = A_t F_t + Pi (F_t + F_s) / 4,
//   A = P g / rho^2, F = dW/dr / r, Pi the viscosity (src/fluid_force.cpp:66-80,89-106).
// Adds to at (t-side inputs) and as (s-side inputs) the gradient of
//   L = abar_t . (m_s r Q) + dubar_t m_s vr S;  alpha_bar gets dL / d alpha.
template <int D, int K, typename T>
SPH_HD void fluid_pair_vjp(const T* rv, const FluidSide<T>& t, const FluidSide<T>& s, T alpha,
                           SideAdj<T>& at, SideAdj<T>& as, T& alpha_bar)
{
    using KF = sphkd::KD<D, K, T>;
    T r2 = T(0);
    for (int k = 0; k < D; ++k) r2 += rv[k] * rv[k];
    const T r = sqrt(r2);
    const T rinv = T(1) / r;
    const T Ft = KF::F(r, t.h), Fs = KF::F(r, s.h);
    const T Frt = KF::F_r(r, t.h), Frs = KF::F_r(r, s.h);
    const T Fht = KF::F_h(r, t.h), Fhs = KF::F_h(r, s.h);
    const T At = t.P * t.g / (t.rho * t.rho), As = s.P * s.g / (s.rho * s.rho);
    T vts[3] = {T(0), T(0), T(0)};
    T vr = T(0);
    for (int k = 0; k < D; ++k) { vts[k] = t.v[k] - s.v[k]; vr += vts[k] * rv[k]; }
    T Pi = T(0), w = T(0), Bb = T(0), vs = T(0), Rr = T(0);
    const bool visc = vr < T(0);
    if (visc) {
        w = vr * rinv;
        Bb = T(0.5) * (t.B + s.B);
        vs = t.c + s.c - T(3) * w;
        Rr = T(2) / (t.rho + s.rho);
        Pi = T(-0.5) * Bb * alpha * vs * w * Rr;
    }
    const T Fsum = Ft + Fs;
    const T Q = -(Ft * At + Fs * As + T(0.5) * Pi * Fsum);
    const T S = At * Ft + T(0.25) * Pi * Fsum;
    T gr = T(0);
    for (int k = 0; k < D; ++k) gr += t.abar[k] * rv[k];
    const T cQ = s.m * gr;
    const T cS = s.m * t.dubar * vr;
    T rvbar[3] = {T(0), T(0), T(0)};
    for (int k = 0; k < D; ++k) rvbar[k] = s.m * Q * t.abar[k];
    T vrbar = s.m * t.dubar * S;
    const T Ftbar = cQ * -(At + T(0.5) * Pi) + cS * (At + T(0.25) * Pi);
    const T Fsbar = cQ * -(As + T(0.5) * Pi) + cS * (T(0.25) * Pi);
    const T Atbar = (cS - cQ) * Ft;
    const T Asbar = -cQ * Fs;
    const T Pibar = (T(-0.5) * cQ + T(0.25) * cS) * Fsum;
    T rbar = T(0);
    if (visc) {
        const T dPi_dw = T(-0.5) * Bb * alpha * Rr * (vs - T(3) * w);
        const T wbar = Pibar * dPi_dw;
        const T Bbbar = Pibar * (T(-0.5) * alpha * vs * w * Rr);
        alpha_bar += Pibar * (T(-0.5) * Bb * vs * w * Rr);
        const T Rrbar = Pibar * (T(-0.5) * Bb * alpha * vs * w);
        const T cbar = Pibar * (T(-0.5) * Bb * alpha * w * Rr);
        const T rhob = Rrbar * (T(-0.5) * Rr * Rr);
        at.B += T(0.5) * Bbbar; as.B += T(0.5) * Bbbar;
        at.rho += rhob; as.rho += rhob;
        at.c += cbar; as.c += cbar;
        vrbar += wbar * rinv;
        rbar -= wbar * vr * rinv * rinv;
    }
    rbar += Ftbar * Frt + Fsbar * Frs;
    at.h += Ftbar * Fht;
    as.h += Fsbar * Fhs;
    at.P += Atbar * t.g / (t.rho * t.rho);
    at.g += Atbar * t.P / (t.rho * t.rho);
    at.rho += Atbar * (T(-2) * At / t.rho);
    as.P += Asbar * s.g / (s.rho * s.rho);
    as.g += Asbar * s.P / (s.rho * s.rho);
    as.rho += Asbar * (T(-2) * As / s.rho);
    for (int k = 0; k < D; ++k) {
        const T vb = vrbar * rv[k];
        rvbar[k] += vrbar * vts[k] + rbar * rv[k] * rinv;
        at.x[k] += rvbar[k];
        as.x[k] -= rvbar[k];
        at.v[k] += vb;
        as.v[k] -= vb;
    }
}

// Sums of one particle over its neighbour set {r < h} that the local backward needs.
// Pressure-energy form: the Balsara sums carry the weight m u instead of m, and
//   n = sum W, n_h, n_hh;  Y_h = sum m u dW/dh, Y_hh  (P = (gamma - 1) sum m u W).
template <typename T>
struct PreSums {
    T rho_h, rho_hh;   // sum m dW/dh, sum m d2W/dh2
    T Dv, Dv_h;        // sum m (v_ij . r_ij) F and its h derivative   (div v = -Dv / rho)
    T Rt[3], Rt_h[3];  // sum m F (v_ij x r_ij) and its h derivative   (rot v = Rt / rho; 2D in [0])
    T n, n_h, n_hh, Y_h, Y_hh;
    SPH_HD void zero()
    {
        rho_h = rho_hh = Dv = Dv_h = T(0);
        n = n_h = n_hh = Y_h = Y_hh = T(0);
        for (int k = 0; k < 3; ++k) { Rt[k] = T(0); Rt_h[k] = T(0); }
    }
};

// cross product r x v as the reference's vector_product: a scalar (z) in 2D, a vector in 3D
template <int D, typename T>
SPH_HD void cross_of(const T* a, const T* b, T* out)
{
    if (D == 2) { out[0] = a[0] * b[1] - a[1] * b[0]; out[1] = T(0); out[2] = T(0); }
    else if (D == 3) {
        out[0] = a[1] * b[2] - a[2] * b[1];
        out[1] = a[2] * b[0] - a[0] * b[2];
        out[2] = a[0] * b[1] - a[1] * b[0];
    } else { out[0] = out[1] = out[2] = T(0); }
}

// Accumulate one pair (j in i's set {r < h_i}, j == i allowed) into i's sums.
template <int D, int K, typename T>
SPH_HD void pre_sums_add(PreSums<T>& ps, const T* rv, const T* vij, T mj, T h)
{
    using KF = sphkd::KD<D, K, T>;
    T r2 = T(0), vr = T(0);
    for (int k = 0; k < D; ++k) { r2 += rv[k] * rv[k]; vr += vij[k] * rv[k]; }
    const T r = sqrt(r2);
    ps.rho_h += mj * KF::w_h(r, h);
    ps.rho_hh += mj * KF::w_hh(r, h);
    if (r == T(0)) return;
    const T F = KF::F(r, h), Fh = KF::F_h(r, h);
    ps.Dv += mj * vr * F;
    ps.Dv_h += mj * vr * Fh;
    T cr[3];
    cross_of<D, T>(vij, rv, cr);
    for (int k = 0; k < 3; ++k) { ps.Rt[k] += mj * F * cr[k]; ps.Rt_h[k] += mj * Fh * cr[k]; }
}

// Weights of a particle's density-type sums in the position / velocity gradients.
template <typename T>
struct PreWeights {
    T w_rho;      // weight of sum m W   (adjoint of rho plus the implicit-h term)
    T w_rhoh;     // weight of sum m dW/dh
    T Dbar;       // weight of Dv
    T Rtbar[3];   // weight of Rt
    T w_n, w_nh, w_Y, w_Yh;   // pressure-energy form: weights of sum W, W_h, m u W, m u W_h
};

// From the adjoints of rho, P, g, h, c, B of one particle (forward values rho, h, c, u and its
// sums) to its sum weights and the adjoint of u (through P and c).  balsara: the switch was
// computed (useBalsaraSwitch and D > 1).
template <int D, typename T>
SPH_HD void pre_local_backward(T rho, T h, T c, T u, T gamma, bool balsara, const PreSums<T>& ps,
                               T rhobar, T Pbar, T gbar, T hbar, T cbar, T Bbar,
                               PreWeights<T>& out, T& ubar)
{
    out.Dbar = T(0);
    out.w_n = out.w_nh = out.w_Y = out.w_Yh = T(0);
    for (int k = 0; k < 3; ++k) out.Rtbar[k] = T(0);
    if (balsara && D > 1) {
        const T div = -ps.Dv / rho;
        T rot[3];
        for (int k = 0; k < 3; ++k) rot[k] = ps.Rt[k] / rho;
        const T rotabs = D == 2 ? fabs(rot[0]) : sqrt(rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2]);
        const T e = T(1e-4) * c / h;
        const T n = fabs(div);
        const T d = n + rotabs + e;
        const T nbar = Bbar * (rotabs + e) / (d * d);
        const T qbar = -Bbar * n / (d * d);
        const T divbar = div > T(0) ? nbar : div < T(0) ? -nbar : T(0);
        T rotbar[3] = {T(0), T(0), T(0)};
        if (D == 2) rotbar[0] = rot[0] > T(0) ? qbar : rot[0] < T(0) ? -qbar : T(0);
        else if (rotabs > T(0)) for (int k = 0; k < 3; ++k) rotbar[k] = qbar * rot[k] / rotabs;
        cbar += qbar * T(1e-4) / h;
        hbar += qbar * (T(-1e-4) * c / (h * h));
        out.Dbar = -divbar / rho;
        rhobar += divbar * ps.Dv / (rho * rho);
        for (int k = 0; k < 3; ++k) {
            out.Rtbar[k] = rotbar[k] / rho;
            rhobar -= rotbar[k] * ps.Rt[k] / (rho * rho);
        }
        hbar += out.Dbar * ps.Dv_h;
        for (int k = 0; k < 3; ++k) hbar += out.Rtbar[k] * ps.Rt_h[k];
    }
    // P = (gamma - 1) rho u
    rhobar += (gamma - T(1)) * u * Pbar;
    ubar = (gamma - T(1)) * rho * Pbar;
    // g = 1 / s, s = 1 + h rho_h / (D rho)
    const T g = T(1) / (T(1) + h * ps.rho_h / (T(D) * rho));
    const T sbar = -g * g * gbar;
    hbar += sbar * ps.rho_h / (T(D) * rho);
    const T rhohbar = sbar * h / (T(D) * rho);
    rhobar -= sbar * h * ps.rho_h / (T(D) * rho * rho);
    // explicit h dependence of the sums rho_h and rho
    hbar += rhohbar * ps.rho_hh;
    hbar += rhobar * ps.rho_h;
    // implicit h: F(h, x) = rho(h, x) h^D - b = 0
    const T hD = sphkd::ipow<D>(h);
    const T hD1 = D == 1 ? T(1) : D == 2 ? h : h * h;
    const T Fh = ps.rho_h * hD + T(D) * rho * hD1;
    const T lambda = -hbar * hD / Fh;
    out.w_rho = rhobar + lambda;
    out.w_rhoh = rhohbar;
    // c = sqrt(gamma (gamma - 1) u)
    ubar += cbar * gamma * (gamma - T(1)) / (T(2) * c);
}

// Position and velocity gradient of the pair (i, j) in the sum of particle `a` (a = i with
// weights wa and smoothing length ha, partner mass mb): rv = x_i - x_j, vij = v_i - v_j.  The same
// expression serves j's sum (a = j, mb = m_i), because the pair terms of the density-type sums
// are even in (r_ij, v_ij).
template <int D, int K, typename T>
SPH_HD void pre_pair_gather(const T* rv, const T* vij, T mb, T ha, const PreWeights<T>& wa,
                            T* xbar, T* vbar)
{
    using KF = sphkd::KD<D, K, T>;
    T r2 = T(0), vr = T(0);
    for (int k = 0; k < D; ++k) { r2 += rv[k] * rv[k]; vr += vij[k] * rv[k]; }
    if (r2 == T(0)) return;
    const T r = sqrt(r2), rinv = T(1) / r;
    const T F = KF::F(r, ha), Fr = KF::F_r(r, ha), Fh = KF::F_h(r, ha);
    // sum m W and sum m dW/dh: d/dx_i = m (F, F_h) r_ij
    const T cw = mb * (wa.w_rho * F + wa.w_rhoh * Fh);
    // Dv = sum m vr F
    const T cd = wa.Dbar * mb;
    // Rt = sum m F (v x r): d/dr = F_r r^ (Rtbar . (v x r)) + F (Rtbar x v);  d/dv = F (r x Rtbar)
    T cr[3];
    cross_of<D, T>(vij, rv, cr);
    T rt = T(0);
    for (int k = 0; k < 3; ++k) rt += wa.Rtbar[k] * cr[k];
    T rbv[3] = {T(0), T(0), T(0)}, rvb[3] = {T(0), T(0), T(0)};
    if (D == 2) {
        // Rtbar along z: Rtbar x v = Rtbar (-v_y, v_x),  r x Rtbar = Rtbar (r_y, -r_x)
        rbv[0] = -wa.Rtbar[0] * vij[1]; rbv[1] = wa.Rtbar[0] * vij[0];
        rvb[0] = wa.Rtbar[0] * rv[1];   rvb[1] = -wa.Rtbar[0] * rv[0];
    } else if (D == 3) {
        cross_of<D, T>(wa.Rtbar, vij, rbv);
        cross_of<D, T>(rv, wa.Rtbar, rvb);
    }
    for (int k = 0; k < D; ++k) {
        xbar[k] += cw * rv[k];
        xbar[k] += cd * (vij[k] * F + vr * Fr * rv[k] * rinv);
        vbar[k] += cd * F * rv[k];
        xbar[k] += mb * (Fr * rinv * rt * rv[k] + F * rbv[k]);
        vbar[k] += mb * F * rvb[k];
    }
}

// ---- fused forms for the device passes ----------------------------------------------------------

// Kernel values of one side of a pair (r > 0) from a single evaluation of the kernel shape:
// F = dW/dr / r, F_r = dF/dr, F_h = dF/dh, W_h = dW/dh, W_hh = d2W/dh2 (kderiv.cuh).
// s = scale(h) (h / 2 for the cubic spline, h for C4), sinv = 1 / s, hinv = 1 / h.
template <typename T>
struct KVals {
    T F, Fr, Fh, W, Wh, Whh;
};

template <int D, int K, typename T, bool WITH_H>
SPH_HD void kvals(T r, T rinv, T s, T sinv, T hinv, KVals<T>& o)
{
    using KF = sphkd::KD<D, K, T>;
    const T q = r * sinv;
    T w0, w1, w2;
    sphkd::shape<K, T>(q, w0, w1, w2);
    const T cD = KF::sig() * sphkd::ipow<D>(sinv);   // sigma / s^D
    const T c2 = cD * sinv * sinv;                     // sigma / s^(D+2)
    const T qinv = s * rinv;
    const T g = w1 * qinv;                             // omega' / q
    o.F = c2 * g;
    o.Fr = c2 * sinv * (w2 - g) * qinv;
    if (WITH_H) {
        o.Fh = -c2 * (T(D + 1) * g + w2) * hinv;
        const T chi = T(D) * w0 + q * w1;
        const T chi1 = T(D + 1) * w1 + q * w2;
        o.W = cD * w0;
        o.Wh = -cD * chi * hinv;
        o.Whh = cD * (T(D + 1) * chi + q * chi1) * hinv * hinv;
    } else {
        o.Fh = o.W = o.Wh = o.Whh = T(0);
    }
}

// One pair (i, j), r_ij != 0, as seen from particle i in the first device pass: adds to i's
// density-type sums (kernel at h_i) and to i's adjoints the part of the two pair terms
// T1 = (target i, source j) and T2 = (target j, source i) of a and du/dt that depends on i's
// inputs.  T1 and T2 share Q = -(F_i X + F_j Y + Pi (F_i + F_j) / 2), so
//   L = cQ Q + c1 S1 + c2 S2,  cQ = (m_j abar_i - m_i abar_j) . r_ij,
//   c1 = m_j dubar_i v_ij . r_ij,  c2 = m_i dubar_j v_ij . r_ij,
//   S1 = X F_i + Pi Fsum / 4,  S2 = Y F_j + Pi Fsum / 4,
// plus the explicit r_ij of the acceleration terms, with
//   standard form (TYPE 0):        X = P_i g_i / rho_i^2,  Y = P_j g_j / rho_j^2
//                                  (src/fluid_force.cpp:66-80);
//   pressure-energy form (TYPE 1): X = (gamma-1)^2 u_i (u_j - g_i / m_j) / P_i,
//                                  Y = (gamma-1)^2 u_j (u_i - g_j / m_i) / P_j
//                                  (src/disph/d_fluid_force.cpp:60-80).
// Every r_ij and v_ij dependence belongs to x_i and v_i; of Pi's symmetric inputs i takes its
// own half.  alpha_bar gets half of the pair's avAlpha adjoint (j's visit adds the other half).
// hinv_j is 1 / h_j.
template <int D, int K, typename T, int TYPE>
SPH_HD void pass1_pair(const T* rv, const T* vij, T r2, const FluidSide<T>& si, const FluidSide<T>& sj,
                       T s_i, T sinv_i, T hinv_i, T hinv_j, T alpha, T gamma,
                       PreSums<T>& ps, SideAdj<T>& mine, T& alpha_bar)
{
    const T rinv = T(1) / sqrt(r2);
    const T r = r2 * rinv;
    KVals<T> ki, kj;
    kvals<D, K, T, true>(r, rinv, s_i, sinv_i, hinv_i, ki);
    const T sinv_j = K == 0 ? T(2) * hinv_j : hinv_j;
    kvals<D, K, T, false>(r, rinv, T(1) / sinv_j, sinv_j, hinv_j, kj);
    T vr = T(0);
    for (int k = 0; k < D; ++k) vr += vij[k] * rv[k];
    // density-type sums of i
    const T mb = TYPE == 1 ? sj.m * sj.u : sj.m;   // weight of the Balsara sums
    ps.rho_h += sj.m * ki.Wh;
    if (TYPE == 0) {
        ps.rho_hh += sj.m * ki.Whh;
    } else {
        ps.n += ki.W;
        ps.n_h += ki.Wh;
        ps.n_hh += ki.Whh;
        ps.Y_h += mb * ki.Wh;
        ps.Y_hh += mb * ki.Whh;
    }
    ps.Dv += mb * vr * ki.F;
    ps.Dv_h += mb * vr * ki.Fh;
    {
        T cr[3];
        cross_of<D, T>(vij, rv, cr);
        for (int k = 0; k < 3; ++k) { ps.Rt[k] += mb * ki.F * cr[k]; ps.Rt_h[k] += mb * ki.Fh * cr[k]; }
    }
    // fluid pair terms
    const T g2 = (gamma - T(1)) * (gamma - T(1));
    T X, Y;
    if (TYPE == 0) {
        X = si.P * si.g / (si.rho * si.rho);
        Y = sj.P * sj.g / (sj.rho * sj.rho);
    } else {
        X = g2 * si.u * (sj.u - si.g / sj.m) / si.P;
        Y = g2 * sj.u * (si.u - sj.g / si.m) / sj.P;
    }
    T Pi = T(0), w = T(0), Bb = T(0), vs = T(0), Rr = T(0);
    const bool visc = vr < T(0);
    if (visc) {
        w = vr * rinv;
        Bb = T(0.5) * (si.B + sj.B);
        vs = si.c + sj.c - T(3) * w;
        Rr = T(2) / (si.rho + sj.rho);
        Pi = T(-0.5) * Bb * alpha * vs * w * Rr;
    }
    const T Fsum = ki.F + kj.F;
    const T Q = -(ki.F * X + kj.F * Y + T(0.5) * Pi * Fsum);
    T dab[3] = {T(0), T(0), T(0)};
    T cQ = T(0);
    for (int k = 0; k < D; ++k) { dab[k] = sj.m * si.abar[k] - si.m * sj.abar[k]; cQ += dab[k] * rv[k]; }
    const T c1 = sj.m * si.dubar * vr, c2 = si.m * sj.dubar * vr;
    const T S1 = X * ki.F + T(0.25) * Pi * Fsum;
    const T S2 = Y * kj.F + T(0.25) * Pi * Fsum;
    const T Fbi = -cQ * (X + T(0.5) * Pi) + c1 * (X + T(0.25) * Pi) + c2 * (T(0.25) * Pi);
    const T Fbj = -cQ * (Y + T(0.5) * Pi) + c1 * (T(0.25) * Pi) + c2 * (Y + T(0.25) * Pi);
    const T Xb = (c1 - cQ) * ki.F;
    const T Pib = (T(-0.5) * cQ + T(0.25) * (c1 + c2)) * Fsum;
    T vrbar = sj.m * si.dubar * S1 + si.m * sj.dubar * S2;
    T rbar = Fbi * ki.Fr + Fbj * kj.Fr;
    mine.h += Fbi * ki.Fh;
    if (visc) {
        const T wbar = Pib * (T(-0.5) * Bb * alpha * Rr * (vs - T(3) * w));
        mine.B += T(0.5) * Pib * (T(-0.5) * alpha * vs * w * Rr);
        alpha_bar += T(0.5) * Pib * (T(-0.5) * Bb * vs * w * Rr);
        const T Rrbar = Pib * (T(-0.5) * Bb * alpha * vs * w);
        mine.c += Pib * (T(-0.5) * Bb * alpha * w * Rr);
        mine.rho += Rrbar * (T(-0.5) * Rr * Rr);
        vrbar += wbar * rinv;
        rbar -= wbar * vr * rinv * rinv;
    }
    if (TYPE == 0) {
        const T rho2i = T(1) / (si.rho * si.rho);
        mine.P += Xb * si.g * rho2i;
        mine.g += Xb * si.P * rho2i;
        mine.rho += Xb * (T(-2) * X / si.rho);
    } else {
        const T Yb = (c2 - cQ) * kj.F;
        mine.u += Xb * g2 * (sj.u - si.g / sj.m) / si.P + Yb * g2 * sj.u / sj.P;
        mine.P -= Xb * X / si.P;
        mine.g -= Xb * g2 * si.u / (sj.m * si.P);
    }
    for (int k = 0; k < D; ++k) {
        mine.x[k] += Q * dab[k] + vrbar * vij[k] + rbar * rv[k] * rinv;
        mine.v[k] += vrbar * rv[k];
    }
}

// The particle's own term (r = 0) of its density-type sums.
template <int D, int K, typename T, int TYPE>
SPH_HD void pre_sums_self(PreSums<T>& ps, T m, T u, T h)
{
    using KF = sphkd::KD<D, K, T>;
    const T Wh = KF::w_h(T(0), h), Whh = KF::w_hh(T(0), h);
    ps.rho_h += m * Wh;
    if (TYPE == 0) {
        ps.rho_hh += m * Whh;
    } else {
        ps.n += KF::w(T(0), h);
        ps.n_h += Wh;
        ps.n_hh += Whh;
        ps.Y_h += m * u * Wh;
        ps.Y_hh += m * u * Whh;
    }
}

// Pressure-energy form (src/disph/d_pre_interaction.cpp:21-230): from the adjoints of rho, P,
// g, h, c, B (and the direct adjoint of u from the force terms) to the weights of the sums
// rho = sum m W, n = sum W, n_h, Y = sum m u W = P / (gamma - 1), Y_h and the Balsara sums, with
//   g = s Y_h / (1 + s n_h), s = h / (D n),  div v = -Dv / Y,  rot v = Rt / Y,
// and the smoothing length as the root of n(h) h^D = N / A (the implicit-h weight goes to the
// number-density sum).  ubar gets the adjoint of u through c and the particle's own term of Y.
template <int D, int K, typename T>
SPH_HD void pre_local_backward_disph(T rho, T h, T c, T u, T P, T m, T gamma, bool balsara,
                                     const PreSums<T>& ps, T rhobar, T Pbar, T gbar, T hbar, T cbar,
                                     T Bbar, PreWeights<T>& out, T& ubar)
{
    using KF = sphkd::KD<D, K, T>;
    (void)rho;
    out.w_rhoh = T(0);
    out.Dbar = T(0);
    for (int k = 0; k < 3; ++k) out.Rtbar[k] = T(0);
    const T Y = P / (gamma - T(1));
    T Ybar = (gamma - T(1)) * Pbar;
    if (balsara && D > 1) {
        const T div = -ps.Dv / Y;
        T rot[3];
        for (int k = 0; k < 3; ++k) rot[k] = ps.Rt[k] / Y;
        const T rotabs = D == 2 ? fabs(rot[0]) : sqrt(rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2]);
        const T e = T(1e-4) * c / h;
        const T nn = fabs(div);
        const T d = nn + rotabs + e;
        const T nbar = Bbar * (rotabs + e) / (d * d);
        const T qbar = -Bbar * nn / (d * d);
        const T divbar = div > T(0) ? nbar : div < T(0) ? -nbar : T(0);
        T rotbar[3] = {T(0), T(0), T(0)};
        if (D == 2) rotbar[0] = rot[0] > T(0) ? qbar : rot[0] < T(0) ? -qbar : T(0);
        else if (rotabs > T(0)) for (int k = 0; k < 3; ++k) rotbar[k] = qbar * rot[k] / rotabs;
        cbar += qbar * T(1e-4) / h;
        hbar += qbar * (T(-1e-4) * c / (h * h));
        out.Dbar = -divbar / Y;
        Ybar += divbar * ps.Dv / (Y * Y);
        for (int k = 0; k < 3; ++k) {
            out.Rtbar[k] = rotbar[k] / Y;
            Ybar -= rotbar[k] * ps.Rt[k] / (Y * Y);
        }
        hbar += out.Dbar * ps.Dv_h;
        for (int k = 0; k < 3; ++k) hbar += out.Rtbar[k] * ps.Rt_h[k];
    }
    // g = t / q, t = s Y_h, q = 1 + s n_h, s = h / (D n)
    const T n = ps.n;
    const T sD = h / (T(D) * n);
    const T q = T(1) + sD * ps.n_h;
    const T t = sD * ps.Y_h;
    const T tbar = gbar / q, qbar = -gbar * t / (q * q);
    const T sbar = tbar * ps.Y_h + qbar * ps.n_h;
    const T Yhbar = tbar * sD, nhbar = qbar * sD;
    hbar += sbar / (T(D) * n);
    T nbar = -sbar * h / (T(D) * n * n);
    // explicit h dependence of the sums
    hbar += rhobar * ps.rho_h + Ybar * ps.Y_h + Yhbar * ps.Y_hh + nbar * ps.n_h + nhbar * ps.n_hh;
    // implicit h: F(h, x) = n(h, x) h^D - b = 0
    const T hD = sphkd::ipow<D>(h);
    const T hD1 = D == 1 ? T(1) : D == 2 ? h : h * h;
    const T Fh = ps.n_h * hD + T(D) * n * hD1;
    const T lambda = -hbar * hD / Fh;
    out.w_rho = rhobar;
    out.w_n = nbar + lambda;
    out.w_nh = nhbar;
    out.w_Y = Ybar;
    out.w_Yh = Yhbar;
    // u: through c = sqrt(gamma (gamma - 1) u) and the own term m u W(0, h) of Y and Y_h
    ubar += cbar * gamma * (gamma - T(1)) / (T(2) * c);
    ubar += m * (Ybar * KF::w(T(0), h) + Yhbar * KF::w_h(T(0), h));
    (void)u;
}

// pre_pair_gather with the kernel values of side a already evaluated (kvals with WITH_H).
template <int D, typename T>
SPH_HD void pre_pair_gather_k(const T* rv, const T* vij, T rinv, T mb, const KVals<T>& ka,
                              const PreWeights<T>& wa, T* xbar, T* vbar)
{
    T vr = T(0);
    for (int k = 0; k < D; ++k) vr += vij[k] * rv[k];
    const T F = ka.F, Fr = ka.Fr, Fh = ka.Fh;
    const T cw = mb * (wa.w_rho * F + wa.w_rhoh * Fh);
    const T cd = wa.Dbar * mb;
    T cr[3];
    cross_of<D, T>(vij, rv, cr);
    T rt = T(0);
    for (int k = 0; k < 3; ++k) rt += wa.Rtbar[k] * cr[k];
    T rbv[3] = {T(0), T(0), T(0)}, rvb[3] = {T(0), T(0), T(0)};
    if (D == 2) {
        rbv[0] = -wa.Rtbar[0] * vij[1]; rbv[1] = wa.Rtbar[0] * vij[0];
        rvb[0] = wa.Rtbar[0] * rv[1];   rvb[1] = -wa.Rtbar[0] * rv[0];
    } else if (D == 3) {
        cross_of<D, T>(wa.Rtbar, vij, rbv);
        cross_of<D, T>(rv, wa.Rtbar, rvb);
    }
    const T cx = cd * vr * Fr * rinv + mb * Fr * rinv * rt;
    for (int k = 0; k < D; ++k) {
        xbar[k] += cw * rv[k] + cd * vij[k] * F + cx * rv[k] + mb * F * rbv[k];
        vbar[k] += cd * F * rv[k] + mb * F * rvb[k];
    }
}

// Pressure-energy form of pre_pair_gather_k: side a's sums hold the partner b with weight
// m_b (rho), 1 (n, n_h) and m_b u_b (Y, Y_h and the Balsara sums).  Adds the position / velocity
// gradient to xbar / vbar and the gradient with respect to the partner's u to ubar_b.
template <int D, typename T>
SPH_HD void pre_pair_gather_disph_k(const T* rv, const T* vij, T rinv, T mb, T ub, const KVals<T>& ka,
                                    const PreWeights<T>& wa, T* xbar, T* vbar, T& ubar_b)
{
    T vr = T(0);
    for (int k = 0; k < D; ++k) vr += vij[k] * rv[k];
    const T F = ka.F, Fr = ka.Fr, Fh = ka.Fh;
    const T mu = mb * ub;
    const T cw = mb * wa.w_rho * F + wa.w_n * F + wa.w_nh * Fh + mu * (wa.w_Y * F + wa.w_Yh * Fh);
    const T cd = wa.Dbar * mu;
    T cr[3];
    cross_of<D, T>(vij, rv, cr);
    T rt = T(0);
    for (int k = 0; k < 3; ++k) rt += wa.Rtbar[k] * cr[k];
    T rbv[3] = {T(0), T(0), T(0)}, rvb[3] = {T(0), T(0), T(0)};
    if (D == 2) {
        rbv[0] = -wa.Rtbar[0] * vij[1]; rbv[1] = wa.Rtbar[0] * vij[0];
        rvb[0] = wa.Rtbar[0] * rv[1];   rvb[1] = -wa.Rtbar[0] * rv[0];
    } else if (D == 3) {
        cross_of<D, T>(wa.Rtbar, vij, rbv);
        cross_of<D, T>(rv, wa.Rtbar, rvb);
    }
    const T cx = cd * vr * Fr * rinv + mu * Fr * rinv * rt;
    for (int k = 0; k < D; ++k) {
        xbar[k] += cw * rv[k] + cd * vij[k] * F + cx * rv[k] + mu * F * rbv[k];
        vbar[k] += cd * F * rv[k] + mu * F * rvb[k];
    }
    ubar_b += mb * (wa.w_Y * ka.W + wa.w_Yh * ka.Wh + wa.Dbar * vr * F + F * rt);
}

}  // namespace sphadj
