// Host check of the adjoint algebra in sphcode_gb300/csrc/adjoint_math.cuh.
//
// A brute-force (all pairs, minimum image) 2D periodic standard-SPH run — smoothing length from
// Newton iterated to round-off, the reference's ssph PreInteraction / FluidForce formulas
// (src/pre_interaction.cpp:39-169, src/fluid_force.cpp:26-106) and the kick-drift-kick leapfrog
// with a fixed dt (src/solver.cpp:431-474) — differentiated in reverse with the functions of
// adjoint_math.cuh, in the same pass structure as the device adjoint (fused sums + fluid VJP, local
// backward, pair gather, leapfrog backward).  adj_check() returns the adjoint directional
// derivatives of L = sum (rho_final - 1)^2 together with central finite differences of the same
// forward map, so that a test can compare them.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../sphcode_gb300/csrc/adjoint_math.cuh"

namespace {

constexpr int D = 2;

struct Run {
    int n = 0;
    int K = 0;
    double m = 0, gamma = 5.0 / 3.0, nnb = 32, dt = 1e-3, alpha = 1.0;
    bool balsara = true;
    int type = 0;   // 0 standard SPH, 1 pressure-energy form
};

struct Pre {
    std::vector<double> h, rho, P, g, B, c;
};

inline double wrap(double d) { return d - floor(d + 0.5); }   // box length 1

void rvec(const std::vector<double>& x, int i, int j, double* r)
{
    for (int k = 0; k < D; ++k) r[k] = wrap(x[i * D + k] - x[j * D + k]);
}

template <int K>
void pre_pass(const Run& R, const std::vector<double>& x, const std::vector<double>& v,
              const std::vector<double>& u, Pre& o)
{
    using KF = sphkd::KD<D, K, double>;
    const int n = R.n;
    o.h.assign(n, 0); o.rho.assign(n, 0); o.P.assign(n, 0); o.g.assign(n, 0); o.B.assign(n, 1); o.c.assign(n, 0);
    // mass density (standard form) or number density (pressure-energy form) times h^D = b
    const double mw = R.type == 1 ? 1.0 : R.m;
    const double b = mw * R.nnb / M_PI;
    for (int i = 0; i < n; ++i) {
        o.c[i] = sqrt(R.gamma * (R.gamma - 1.0) * u[i]);
        double h = sqrt(R.nnb * R.m / M_PI);
        for (int it = 0; it < 60; ++it) {
            double rho = 0, rh = 0;
            for (int j = 0; j < n; ++j) {
                double r[D];
                rvec(x, i, j, r);
                const double rr = sqrt(r[0] * r[0] + r[1] * r[1]);
                rho += mw * KF::w(rr, h);
                rh += mw * KF::w_h(rr, h);
            }
            const double f = rho * h * h - b, df = rh * h * h + 2.0 * rho * h;
            const double dh = f / df;
            h -= dh;
            if (fabs(dh) < 1e-15 * h) break;
        }
        sphadj::PreSums<double> ps;
        ps.zero();
        double rho = 0;
        for (int j = 0; j < n; ++j) {
            double r[D], vij[D];
            rvec(x, i, j, r);
            for (int k = 0; k < D; ++k) vij[k] = v[i * D + k] - v[j * D + k];
            rho += R.m * KF::w(sqrt(r[0] * r[0] + r[1] * r[1]), h);
            sphadj::pre_sums_add<D, K, double>(ps, r, vij, R.m, h);
        }
        o.h[i] = h;
        o.rho[i] = rho;
        if (R.type == 0) {
            o.P[i] = (R.gamma - 1.0) * rho * u[i];
            o.g[i] = 1.0 / (1.0 + h * ps.rho_h / (D * rho));
            if (R.balsara) {
                const double div = -ps.Dv / rho, rot = ps.Rt[0] / rho;
                o.B[i] = fabs(div) / (fabs(div) + fabs(rot) + 1e-4 * o.c[i] / h);
            }
            continue;
        }
        // pressure-energy form (src/disph/d_pre_interaction.cpp:60-154)
        double nd = 0, Ys = 0, Yh = 0, nh = 0, dv = 0, rt = 0;
        for (int j = 0; j < n; ++j) {
            double r[D];
            rvec(x, i, j, r);
            const double rr = sqrt(r[0] * r[0] + r[1] * r[1]);
            const double w = KF::w(rr, h), wh = KF::w_h(rr, h);
            nd += w;
            nh += wh;
            Ys += R.m * u[j] * w;
            Yh += R.m * u[j] * wh;
            if (j == i) continue;
            const double F = KF::F(rr, h);
            const double vx = v[i * D] - v[j * D], vy = v[i * D + 1] - v[j * D + 1];
            dv += R.m * u[j] * (vx * r[0] + vy * r[1]) * F;
            rt += R.m * u[j] * (vx * r[1] - vy * r[0]) * F;
        }
        o.P[i] = (R.gamma - 1.0) * Ys;
        o.g[i] = h / (D * nd) * Yh / (1.0 + h / (D * nd) * nh);
        if (R.balsara) {
            const double div = -dv / Ys, rot = rt / Ys;
            o.B[i] = fabs(div) / (fabs(div) + fabs(rot) + 1e-4 * o.c[i] / h);
        }
    }
}

template <int K>
void fluid_pass(const Run& R, const std::vector<double>& x, const std::vector<double>& v,
                const std::vector<double>& u, const Pre& p, double alpha, std::vector<double>& a,
                std::vector<double>& du)
{
    using KF = sphkd::KD<D, K, double>;
    const int n = R.n;
    a.assign(n * D, 0);
    du.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        const double Ai = p.P[i] * p.g[i] / (p.rho[i] * p.rho[i]);
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double r[D], vij[D];
            rvec(x, i, j, r);
            const double rr = sqrt(r[0] * r[0] + r[1] * r[1]);
            if (rr >= fmax(p.h[i], p.h[j])) continue;
            double vr = 0;
            for (int k = 0; k < D; ++k) { vij[k] = v[i * D + k] - v[j * D + k]; vr += vij[k] * r[k]; }
            const double Fi = KF::F(rr, p.h[i]), Fj = KF::F(rr, p.h[j]);
            const double Aj = p.P[j] * p.g[j] / (p.rho[j] * p.rho[j]);
            double Pi = 0;
            if (vr < 0) {
                const double w = vr / rr;
                Pi = -0.5 * 0.5 * (p.B[i] + p.B[j]) * alpha * (p.c[i] + p.c[j] - 3 * w) * w * 2.0 / (p.rho[i] + p.rho[j]);
            }
            double Xi = Ai, Yj = Aj;
            if (R.type == 1) {
                // src/disph/d_fluid_force.cpp:60-80
                const double g2 = (R.gamma - 1.0) * (R.gamma - 1.0);
                Xi = g2 * u[i] * u[j] * (1.0 - p.g[i] / (R.m * u[j])) / p.P[i];
                Yj = g2 * u[i] * u[j] * (1.0 - p.g[j] / (R.m * u[i])) / p.P[j];
            }
            const double Q = -(Fi * Xi + Fj * Yj + 0.5 * Pi * (Fi + Fj));
            for (int k = 0; k < D; ++k) a[i * D + k] += R.m * r[k] * Q;
            du[i] += R.m * vr * (Xi * Fi + 0.25 * Pi * (Fi + Fj));
        }
    }
}

struct St {
    std::vector<double> x, v, u, a, du;
};

template <int K>
void initialize(const Run& R, St& s, Pre& p, double alpha)
{
    pre_pass<K>(R, s.x, s.v, s.u, p);
    fluid_pass<K>(R, s.x, s.v, s.u, p, alpha, s.a, s.du);
}

template <int K>
void step(const Run& R, St& s, Pre& p, double alpha)
{
    const int n = R.n;
    const double dt = R.dt;
    std::vector<double> vp(n * D), up(n);
    for (int i = 0; i < n * D; ++i) {
        vp[i] = s.v[i] + s.a[i] * 0.5 * dt;
        s.x[i] += vp[i] * dt;
        s.v[i] += s.a[i] * dt;
    }
    for (int i = 0; i < n; ++i) {
        up[i] = s.u[i] + s.du[i] * 0.5 * dt;
        s.u[i] += s.du[i] * dt;
    }
    pre_pass<K>(R, s.x, s.v, s.u, p);
    fluid_pass<K>(R, s.x, s.v, s.u, p, alpha, s.a, s.du);
    for (int i = 0; i < n * D; ++i) s.v[i] = vp[i] + s.a[i] * 0.5 * dt;
    for (int i = 0; i < n; ++i) s.u[i] = up[i] + s.du[i] * 0.5 * dt;
}

template <int K>
double loss(const Run& R, St s, int steps, double alpha)
{
    Pre p;
    initialize<K>(R, s, p, alpha);
    for (int t = 0; t < steps; ++t) step<K>(R, s, p, alpha);
    double L = 0;
    for (int i = 0; i < R.n; ++i) L += (p.rho[i] - 1.0) * (p.rho[i] - 1.0);
    return L;
}

// Backward through Pre and Fluid at (x, v, u): abar / dubar are the adjoints of the fluid outputs,
// rhobar_ext an extra adjoint of the density.  Adds the results to xbar, vbar, ubar; returns the
// alpha adjoint.
template <int K, bool FUSED = true>
double pre_fluid_backward(const Run& R, const std::vector<double>& x, const std::vector<double>& v,
                          const std::vector<double>& u, const Pre& p, double alpha,
                          const std::vector<double>& abar, const std::vector<double>& dubar,
                          const std::vector<double>& rhobar_ext, std::vector<double>& xbar,
                          std::vector<double>& vbar, std::vector<double>& ubar)
{
    const int n = R.n;
    double alpha_bar = 0;
    std::vector<sphadj::PreSums<double>> sums(n);
    std::vector<sphadj::SideAdj<double>> loc(n);
    auto side = [&](int i) {
        sphadj::FluidSide<double> s;
        for (int k = 0; k < 3; ++k) { s.v[k] = k < D ? v[i * D + k] : 0; s.abar[k] = k < D ? abar[i * D + k] : 0; }
        s.rho = p.rho[i]; s.P = p.P[i]; s.g = p.g[i]; s.B = p.B[i]; s.c = p.c[i]; s.h = p.h[i]; s.m = R.m;
        s.u = u[i];
        s.dubar = dubar[i];
        return s;
    };
    // pass 1: sums and the fluid VJP in both directions
    for (int i = 0; i < n; ++i) {
        sums[i].zero();
        loc[i].zero();
        const sphadj::FluidSide<double> si = side(i);
        for (int j = 0; j < n; ++j) {
            double r[3] = {0, 0, 0}, vij[3] = {0, 0, 0};
            rvec(x, i, j, r);
            for (int k = 0; k < D; ++k) vij[k] = v[i * D + k] - v[j * D + k];
            if (FUSED && j == i) {
                if (R.type == 0) sphadj::pre_sums_self<D, K, double, 0>(sums[i], R.m, u[i], p.h[i]);
                else sphadj::pre_sums_self<D, K, double, 1>(sums[i], R.m, u[i], p.h[i]);
                continue;
            }
            if (FUSED) {
                const sphadj::FluidSide<double> sj = side(j);
                const double s_i = K == 0 ? 0.5 * p.h[i] : p.h[i];
                const double r2 = r[0] * r[0] + r[1] * r[1];
                if (R.type == 0)
                    sphadj::pass1_pair<D, K, double, 0>(r, vij, r2, si, sj, s_i, 1.0 / s_i, 1.0 / p.h[i],
                                                        1.0 / p.h[j], alpha, R.gamma, sums[i], loc[i], alpha_bar);
                else
                    sphadj::pass1_pair<D, K, double, 1>(r, vij, r2, si, sj, s_i, 1.0 / s_i, 1.0 / p.h[i],
                                                        1.0 / p.h[j], alpha, R.gamma, sums[i], loc[i], alpha_bar);
                continue;
            }
            sphadj::pre_sums_add<D, K, double>(sums[i], r, vij, R.m, p.h[i]);
            if (j == i) continue;
            const sphadj::FluidSide<double> sj = side(j);
            sphadj::SideAdj<double> dummy;
            dummy.zero();
            sphadj::fluid_pair_vjp<D, K, double>(r, si, sj, alpha, loc[i], dummy, alpha_bar);
            double rji[3] = {-r[0], -r[1], 0};
            double ab_unused = 0;
            sphadj::fluid_pair_vjp<D, K, double>(rji, sj, si, alpha, dummy, loc[i], ab_unused);
        }
    }
    // local backward
    std::vector<sphadj::PreWeights<double>> W(n);
    for (int i = 0; i < n; ++i) {
        double ub = loc[i].u;
        if (R.type == 0)
            sphadj::pre_local_backward<D, double>(p.rho[i], p.h[i], p.c[i], u[i], R.gamma, R.balsara, sums[i],
                                                  loc[i].rho + rhobar_ext[i], loc[i].P, loc[i].g, loc[i].h,
                                                  loc[i].c, loc[i].B, W[i], ub);
        else
            sphadj::pre_local_backward_disph<D, K, double>(p.rho[i], p.h[i], p.c[i], u[i], p.P[i], R.m, R.gamma,
                                                           R.balsara, sums[i], loc[i].rho + rhobar_ext[i],
                                                           loc[i].P, loc[i].g, loc[i].h, loc[i].c, loc[i].B,
                                                           W[i], ub);
        ubar[i] += ub;
        for (int k = 0; k < D; ++k) { xbar[i * D + k] += loc[i].x[k]; vbar[i * D + k] += loc[i].v[k]; }
    }
    // pass 2: gather of the density-type sums' derivatives
    for (int i = 0; i < n; ++i) {
        double xb[3] = {0, 0, 0}, vb[3] = {0, 0, 0};
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double r[3] = {0, 0, 0}, vij[3] = {0, 0, 0};
            rvec(x, i, j, r);
            for (int k = 0; k < D; ++k) vij[k] = v[i * D + k] - v[j * D + k];
            if (FUSED) {
                const double rr = sqrt(r[0] * r[0] + r[1] * r[1]), rinv = 1.0 / rr;
                sphadj::KVals<double> ki, kj;
                const double si_ = K == 0 ? 0.5 * p.h[i] : p.h[i], sj_ = K == 0 ? 0.5 * p.h[j] : p.h[j];
                sphadj::kvals<D, K, double, true>(rr, rinv, si_, 1.0 / si_, 1.0 / p.h[i], ki);
                sphadj::kvals<D, K, double, true>(rr, rinv, sj_, 1.0 / sj_, 1.0 / p.h[j], kj);
                if (R.type == 0) {
                    sphadj::pre_pair_gather_k<D, double>(r, vij, rinv, R.m, ki, W[i], xb, vb);
                    sphadj::pre_pair_gather_k<D, double>(r, vij, rinv, R.m, kj, W[j], xb, vb);
                } else {
                    double u_unused = 0;
                    sphadj::pre_pair_gather_disph_k<D, double>(r, vij, rinv, R.m, u[j], ki, W[i], xb, vb, u_unused);
                    sphadj::pre_pair_gather_disph_k<D, double>(r, vij, rinv, R.m, u[i], kj, W[j], xb, vb, ubar[i]);
                }
                continue;
            }
            sphadj::pre_pair_gather<D, K, double>(r, vij, R.m, p.h[i], W[i], xb, vb);
            sphadj::pre_pair_gather<D, K, double>(r, vij, R.m, p.h[j], W[j], xb, vb);
        }
        for (int k = 0; k < D; ++k) { xbar[i * D + k] += xb[k]; vbar[i * D + k] += vb[k]; }
    }
    return alpha_bar;
}

template <int K>
void gradient(const Run& R, const St& s0, int steps, double alpha, std::vector<double>& gv,
              double& galpha, std::vector<double>& gu)
{
    const int n = R.n;
    const double dt = R.dt;
    // forward, keeping every state
    std::vector<St> S(steps + 1);
    Pre p;
    S[0] = s0;
    initialize<K>(R, S[0], p, alpha);
    for (int t = 0; t < steps; ++t) {
        S[t + 1] = S[t];
        step<K>(R, S[t + 1], p, alpha);
    }
    std::vector<double> rhobar(n);
    for (int i = 0; i < n; ++i) rhobar[i] = 2.0 * (p.rho[i] - 1.0);
    std::vector<double> xb(n * D, 0), vb(n * D, 0), ub(n, 0), ab(n * D, 0), dub(n, 0);
    galpha = 0;
    std::vector<double> zero(n, 0);
    for (int t = steps - 1; t >= 0; --t) {
        // recompute the post-predict state of step t
        const St& s = S[t];
        std::vector<double> x1(n * D), v1(n * D), u1(n);
        for (int i = 0; i < n * D; ++i) {
            x1[i] = s.x[i] + (s.v[i] + s.a[i] * 0.5 * dt) * dt;
            v1[i] = s.v[i] + s.a[i] * dt;
        }
        for (int i = 0; i < n; ++i) u1[i] = s.u[i] + s.du[i] * dt;
        Pre q;
        pre_pass<K>(R, x1, v1, u1, q);
        std::vector<double> abt(n * D), dubt(n);
        for (int i = 0; i < n * D; ++i) abt[i] = ab[i] + vb[i] * 0.5 * dt;
        for (int i = 0; i < n; ++i) dubt[i] = dub[i] + ub[i] * 0.5 * dt;
        std::vector<double> x1b(xb), v1b(n * D, 0), u1b(n, 0);
        galpha += pre_fluid_backward<K>(R, x1, v1, u1, q, alpha, abt, dubt, t == steps - 1 ? rhobar : zero,
                                        x1b, v1b, u1b);
        std::vector<double> nxb(n * D), nvb(n * D), nab(n * D), nub(n), ndub(n);
        for (int i = 0; i < n * D; ++i) {
            const double vpb = vb[i] + x1b[i] * dt;
            nxb[i] = x1b[i];
            nvb[i] = v1b[i] + vpb;
            nab[i] = v1b[i] * dt + vpb * 0.5 * dt;
        }
        for (int i = 0; i < n; ++i) {
            const double upb = ub[i];
            nub[i] = u1b[i] + upb;
            ndub[i] = u1b[i] * dt + upb * 0.5 * dt;
        }
        xb.swap(nxb); vb.swap(nvb); ab.swap(nab); ub.swap(nub); dub.swap(ndub);
    }
    // initialize: a0, du0 from Pre and Fluid at the initial state
    {
        Pre q;
        pre_pass<K>(R, s0.x, s0.v, s0.u, q);
        galpha += pre_fluid_backward<K>(R, s0.x, s0.v, s0.u, q, alpha, ab, dub, steps == 0 ? rhobar : zero,
                                        xb, vb, ub);
    }
    gv = vb;
    gu = ub;
}

template <int K>
void check(int side, int steps, double eps, int balsara, double vnoise, int type, double* out)
{
    Run R;
    R.type = type;
    R.balsara = balsara != 0;
    R.K = K;
    R.n = side * side;
    R.m = 1.0 / R.n;
    R.nnb = 32;
    R.dt = 2e-3;
    St s;
    uint64_t z = 12345;
    auto rnd = [&]() {
        z = z * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    s.x.resize(R.n * D); s.v.resize(R.n * D); s.u.resize(R.n);
    for (int i = 0; i < R.n; ++i) {
        const double px = -0.5 + ((i % side) + 0.5 + 0.1 * (rnd() - 0.5)) / side;
        const double py = -0.5 + ((i / side) + 0.5 + 0.1 * (rnd() - 0.5)) / side;
        s.x[i * D] = px; s.x[i * D + 1] = py;
        const double r = sqrt(px * px + py * py);
        const double vphi = r < 0.2 ? 5 * r : r < 0.4 ? 2 - 5 * r : 0;
        s.v[i * D] = (r > 0 ? -py / r * vphi : 0) + vnoise * (rnd() - 0.5);
        s.v[i * D + 1] = (r > 0 ? px / r * vphi : 0) + vnoise * (rnd() - 0.5);
        s.u[i] = (5.0 + 12.5 * r * r + 0.3 * rnd()) / ((R.gamma - 1.0) * 1.0);
    }
    std::vector<double> dv(R.n * D), du(R.n);
    for (auto& q : dv) q = rnd() - 0.5;
    for (auto& q : du) q = rnd() - 0.5;
    std::vector<double> gv, gu;
    double ga;
    gradient<K>(R, s, steps, R.alpha, gv, ga, gu);
    double adj_v = 0, adj_u = 0;
    for (int i = 0; i < R.n * D; ++i) adj_v += gv[i] * dv[i];
    for (int i = 0; i < R.n; ++i) adj_u += gu[i] * du[i];
    auto shifted = [&](double sv, double su) {
        St t = s;
        for (int i = 0; i < R.n * D; ++i) t.v[i] += sv * dv[i];
        for (int i = 0; i < R.n; ++i) t.u[i] += su * du[i];
        return t;
    };
    const double fd_v = (loss<K>(R, shifted(eps, 0), steps, R.alpha) - loss<K>(R, shifted(-eps, 0), steps, R.alpha)) / (2 * eps);
    const double fd_u = (loss<K>(R, shifted(0, eps), steps, R.alpha) - loss<K>(R, shifted(0, -eps), steps, R.alpha)) / (2 * eps);
    const double fd_a = (loss<K>(R, s, steps, R.alpha + eps) - loss<K>(R, s, steps, R.alpha - eps)) / (2 * eps);
    out[0] = adj_v; out[1] = fd_v;
    out[2] = adj_u; out[3] = fd_u;
    out[4] = ga;    out[5] = fd_a;
    out[6] = loss<K>(R, s, steps, R.alpha);
}

// One Pre + Fluid evaluation: L = ca . a + cdu . du + crho . rho, gradient in x, v, u along
// random directions by the adjoint and by central differences.
template <int K>
void check_single(int side, double eps, int balsara, int which, int type, double* out)
{
    Run R;
    R.K = K;
    R.type = type;
    R.balsara = balsara != 0;
    R.n = side * side;
    R.m = 1.0 / R.n;
    uint64_t z = 777;
    auto rnd = [&]() {
        z = z * 6364136223846793005ULL + 1442695040888963407ULL;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    St s;
    s.x.resize(R.n * D); s.v.resize(R.n * D); s.u.resize(R.n);
    for (int i = 0; i < R.n; ++i) {
        s.x[i * D] = -0.5 + ((i % side) + 0.5 + 0.2 * (rnd() - 0.5)) / side;
        s.x[i * D + 1] = -0.5 + ((i / side) + 0.5 + 0.2 * (rnd() - 0.5)) / side;
        s.v[i * D] = rnd() - 0.5;
        s.v[i * D + 1] = rnd() - 0.5;
        s.u[i] = 1.0 + rnd();
    }
    std::vector<double> ca(R.n * D), cdu(R.n), crho(R.n);
    for (auto& q : ca) q = (which & 1) ? rnd() - 0.5 : 0.0;
    for (auto& q : cdu) q = (which & 2) ? rnd() - 0.5 : 0.0;
    for (auto& q : crho) q = (which & 4) ? rnd() - 0.5 : 0.0;
    auto L = [&](const St& t) {
        Pre p;
        std::vector<double> a, du;
        pre_pass<K>(R, t.x, t.v, t.u, p);
        fluid_pass<K>(R, t.x, t.v, t.u, p, R.alpha, a, du);
        double l = 0;
        for (int i = 0; i < R.n * D; ++i) l += ca[i] * a[i];
        for (int i = 0; i < R.n; ++i) l += cdu[i] * du[i] + crho[i] * p.rho[i];
        return l;
    };
    Pre p;
    pre_pass<K>(R, s.x, s.v, s.u, p);
    std::vector<double> xb(R.n * D, 0), vb(R.n * D, 0), ub(R.n, 0);
    const double ab = pre_fluid_backward<K>(R, s.x, s.v, s.u, p, R.alpha, ca, cdu, crho, xb, vb, ub);
    {
        // the fused device forms against the two-call forms
        std::vector<double> xb2(R.n * D, 0), vb2(R.n * D, 0), ub2(R.n, 0);
        // the two-call forms exist for the standard form only
        const double ab2 = R.type != 0 ? ab : pre_fluid_backward<K, false>(R, s.x, s.v, s.u, p, R.alpha, ca, cdu,
                                                                           crho, xb2, vb2, ub2);
        if (R.type != 0) { xb2 = xb; vb2 = vb; ub2 = ub; }
        double d = fabs(ab - ab2) / (fabs(ab2) + 1e-300), mx = 0, mv = 0, mu = 0;
        for (int i = 0; i < R.n * D; ++i) { mx = fmax(mx, fabs(xb2[i])); mv = fmax(mv, fabs(vb2[i])); }
        for (int i = 0; i < R.n; ++i) mu = fmax(mu, fabs(ub2[i]));
        for (int i = 0; i < R.n * D; ++i) { d = fmax(d, fabs(xb[i] - xb2[i]) / mx); d = fmax(d, fabs(vb[i] - vb2[i]) / mv); }
        for (int i = 0; i < R.n; ++i) d = fmax(d, fabs(ub[i] - ub2[i]) / (mu + 1e-300));
        out[6] = d;
    }
    std::vector<double> dx(R.n * D), dv(R.n * D), du(R.n);
    for (auto& q : dx) q = rnd() - 0.5;
    for (auto& q : dv) q = rnd() - 0.5;
    for (auto& q : du) q = rnd() - 0.5;
    double gx = 0, gv = 0, gu = 0;
    for (int i = 0; i < R.n * D; ++i) { gx += xb[i] * dx[i]; gv += vb[i] * dv[i]; }
    for (int i = 0; i < R.n; ++i) gu += ub[i] * du[i];
    auto sh = [&](int f, double e) {
        St t = s;
        if (f == 0) for (int i = 0; i < R.n * D; ++i) t.x[i] += e * dx[i];
        if (f == 1) for (int i = 0; i < R.n * D; ++i) t.v[i] += e * dv[i];
        if (f == 2) for (int i = 0; i < R.n; ++i) t.u[i] += e * du[i];
        return t;
    };
    out[0] = gx; out[1] = (L(sh(0, eps)) - L(sh(0, -eps))) / (2 * eps);
    out[2] = gv; out[3] = (L(sh(1, eps)) - L(sh(1, -eps))) / (2 * eps);
    out[4] = gu; out[5] = (L(sh(2, eps)) - L(sh(2, -eps))) / (2 * eps);
}

// Gradient of L = sum (rho_final - 1)^2 for given initial fields (n particles of mass 1/n in the
// periodic unit box [-0.5, 0.5)^2, gamma 5/3): gv (n*2), gu (n), *galpha, and rho_final (n).
template <int K>
void gradient_of(int n, int steps, double dt, double alpha, double nnb, int balsara, int type, const double* x,
                 const double* v, const double* u, double* gv_out, double* gu_out, double* galpha,
                 double* rho_out)
{
    Run R;
    R.type = type;
    R.K = K;
    R.n = n;
    R.m = 1.0 / n;
    R.nnb = nnb;
    R.dt = dt;
    R.alpha = alpha;
    R.balsara = balsara != 0;
    St s;
    s.x.assign(x, x + n * D);
    s.v.assign(v, v + n * D);
    s.u.assign(u, u + n);
    std::vector<double> gv, gu;
    gradient<K>(R, s, steps, alpha, gv, *galpha, gu);
    for (int i = 0; i < n * D; ++i) gv_out[i] = gv[i];
    for (int i = 0; i < n; ++i) gu_out[i] = gu[i];
    St f = s;
    Pre p;
    initialize<K>(R, f, p, alpha);
    for (int t = 0; t < steps; ++t) step<K>(R, f, p, alpha);
    for (int i = 0; i < n; ++i) rho_out[i] = p.rho[i];
}

}  // namespace

extern "C" void adj_gradient(int kernel, int type, int n, int steps, double dt, double alpha, double nnb,
                             int balsara, const double* x, const double* v, const double* u, double* gv,
                             double* gu, double* galpha, double* rho)
{
    if (kernel == 0) gradient_of<0>(n, steps, dt, alpha, nnb, balsara, type, x, v, u, gv, gu, galpha, rho);
    else gradient_of<1>(n, steps, dt, alpha, nnb, balsara, type, x, v, u, gv, gu, galpha, rho);
}

extern "C" void adj_check_single(int kernel, int type, int side, double eps, int balsara, int which, double* out)
{
    if (kernel == 0) check_single<0>(side, eps, balsara, which, type, out);
    else check_single<1>(side, eps, balsara, which, type, out);
}

// out[7]: adjoint / finite-difference pairs for a velocity direction, an energy direction and
// avAlpha, then the loss.  kernel 0 cubic spline, 1 Wendland C4.
extern "C" void adj_check(int kernel, int type, int side, int steps, double eps, int balsara, double vnoise,
                          double* out)
{
    if (kernel == 0) check<0>(side, steps, eps, balsara, vnoise, type, out);
    else check<1>(side, steps, eps, balsara, vnoise, type, out);
}
