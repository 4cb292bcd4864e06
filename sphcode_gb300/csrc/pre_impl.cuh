// PreInteraction on the device: smoothing length by Newton iteration, density, pressure, grad-h
// term, signal velocity, Balsara switch and time-dependent viscosity (ssph:
// src/pre_interaction.cpp:39-169,227-283; disph: src/disph/d_pre_interaction.cpp:21-230) or the
// MUSCL gradients (gsph: src/gsph/g_pre_interaction.cpp:27-144), and the first-call
// initial_smoothing (src/pre_interaction.cpp:171-215).
//
// One CTA per target group (group.cuh).  The candidate set of a target is the reference's:
// {j : r_ij^2 < h_s^2} with h_s = 1.2 h_guess (the search radius of src/pre_interaction.cpp:64,70),
// decided exactly.  Newton iterations and the density loop run over the candidate bitmask with
// the pair terms in T; the reference's `r >= h -> break` over the distance-sorted list is the
// set {r < h}; at the final h that set is decided exactly (it defines the neighbour count).
// The Newton step f / f' is formed from the T sums; h itself and the convergence test
// |dh| < 1e-4 (h + h_prev) stay FP64.
#pragma once

#include "context.cuh"
#include "group.cuh"

namespace sphgpu {

template <typename T>
struct PreArgs {
    using V4 = typename Vec4<T>::type;
    State st;
    TreeView tv;
    Periodic pb;
    SmemLayout L;
    GroupWork work;
    const V4* xrel;                       // {x - leaf centre, m}
    const V4* mvel;                       // {vx, vy, vz, c}
    const T* mu;                          // u
    int nn;
    double ratio;
    double gamma;
    int iterative;
    int initial;
    int use_balsara, use_tdav;
    int gsph_2nd;
    double alpha_min, alpha_max, eps_av;
    const double* dt_run;
    long long* hvs;
    int* newton_fail;
    double* hguess;   // per-particle guess: the first pass stores it, later passes reuse it
    double nn_over_a; // neighborNumber / A_D
    unsigned long long* counters;   // PairCounter slots, or nullptr (not counted)
    int bulk_stage;                 // stage the tile with bulk asynchronous copies (knob 29)
    PlanView<T> pv;                 // group plans of the first pass (pv.plan nullptr: none)
    // inside a whole step (ssph / disph): FluidForce's source records {v, 1/h}, {rho, P, c, X},
    // {alpha, balsara, u, Y} written by each finished target, as fluid_mirror_kernel would form
    // them from the fields this stage stores (nullptr: the mirror kernel runs before FluidForce)
    V4* frec0;
    V4* frec1;
    V4* frec2;
};

template <int D>
__device__ __forceinline__ double h_guess(double nn, double m, double rho)
{
    const double x = nn * m / (rho * volume_const<D>());
    if (D == 1) return x;
    if (D == 2) return sqrt(x);          // = pow(x, 0.5), both correctly rounded
    return pow(x, 1.0 / 3.0);
}

// Pair source of the group schedule: the candidate bits of the target over the CTA's staged
// tile (exact candidates, see pre_kernel); restrict() clears the bits beyond h (T test outside
// the guard band, the reference's FP64 r < h inside it, in a loop of its own) so that the member
// loops run without divergence on non-members.
template <int D, typename T>
struct TilePreSource {
    using V4 = typename Vec4<T>::type;
    const Tile<T>* tile;
    const State* st;
    const Periodic* pb;
    const V4* mvel;
    const double* xi;
    const T* xo;
    int gt, t, nw;
    unsigned long long wmask;
    const GroupMisc* gm;

    template <class F>
    __device__ __forceinline__ void newton_pass(F f)
    {
        MaskWordIter it(tile->mask, gt, t, nw, wmask);
        int sa, sb;
        while (it.next(sa)) {
            const bool two = it.next(sb);
            T r[D];
            const V4 pa = tile->pm[sa];
            const T rra = sqrt(tile_r2<D, T>(xo, pa, r));
            T rrb = T(0), mb = T(0);
            if (two) {
                const V4 pb_ = tile->pm[sb];
                rrb = sqrt(tile_r2<D, T>(xo, pb_, r));
                mb = pb_.w;
            }
            f(rra, pa.w, rrb, mb, two);
        }
    }

    __device__ __forceinline__ void restrict(double hf)
    {
        const double hf2 = __dmul_rn(hf, hf);
        const double band = r2_band<T, D>(gm, hf);
        const T lo_t = to_T_down<T>(hf2 - band), hi_t = to_T_up<T>(hf2 + band);
        bool in_band = false;
        {
            // word by word: two candidates per trip (independent shared loads and tests), one
            // store of the word's remaining bits
            MaskWordIter it(tile->mask, gt, t, nw, wmask);
            int w;
            unsigned cb;
            while (it.next_word(w, cb)) {
                unsigned keep = cb, rem = cb;
                while (rem) {
                    const int b0 = __ffs(rem) - 1;
                    rem &= rem - 1;
                    const int b1 = rem ? __ffs(rem) - 1 : b0;
                    rem &= rem - 1;
                    T r[D];
                    const T r2a = tile_r2<D, T>(xo, tile->pm[w * 32 + b0], r);
                    const T r2b = tile_r2<D, T>(xo, tile->pm[w * 32 + b1], r);
                    if (r2a > hi_t) keep &= ~(1u << b0); else in_band |= !(r2a < lo_t);
                    if (r2b > hi_t) keep &= ~(1u << b1); else in_band |= !(r2b < lo_t);
                }
                if (keep != cb) tile->mask[w * gt + t] = keep;
            }
        }
        if (in_band) {
            MaskWordIter it(tile->mask, gt, t, nw, wmask);
            int s;
            while (it.next(s)) {
                T r[D];
                const T r2 = tile_r2<D, T>(xo, tile->pm[s], r);
                if (!(r2 < lo_t) && !(__dsqrt_rn(exact_r2<D>(*st, xi, tile->idx[s], *pb)) < hf)) it.clear(s);
            }
        }
    }

    template <class F>
    __device__ __forceinline__ void for_members(bool load_v, F f)
    {
        // the next member's velocity record is loaded before the current one is evaluated
        MaskWordIter it(tile->mask, gt, t, nw, wmask);
        int snext;
        bool have = it.next(snext);
        V4 vq{};
        if (have && load_v) vq = mvel[tile->idx[snext]];
        while (have) {
            const int s = snext;
            const V4 vjr = vq;
            have = it.next(snext);
            if (have && load_v) vq = mvel[tile->idx[snext]];
            const V4 p = tile->pm[s];
            T r[D];
            const T r2 = tile_r2<D, T>(xo, p, r);
            f(r, r2, p.w, tile->aux[s], tile->idx[s], vjr);
        }
    }
};

// Pair source of the thread-per-particle schedule: the target's own walk (search radius h_s, the
// reference's BHTree::neighbor_search without is_ij), once per pass; candidates r_ij^2 < h_s^2
// and members r_ij < h decided exactly (T test outside the walker's guard band, the reference's
// FP64 arithmetic inside it).
template <int D, typename T>
struct WalkPreSource {
    using V4 = typename Vec4<T>::type;
    const TreeView* tv;
    const Periodic* pb;
    const State* st;
    const V4* xrel;
    const V4* mvel;
    const T* mu;
    const double* xi;
    double hs, hf;
    int root;
    bool active, restricted;

    // next candidate (or member, once restricted) of the walk w: separation, r^2 and slot
    __device__ __forceinline__ bool next(TargetWalk<D, T>& w, T* r, T& r2, V4& q, int& j)
    {
        const double hs2 = __dmul_rn(hs, hs);
        const T hsT = (T)hs, hfT = (T)hf;
        while (w.next(j)) {
            q = xrel[j];
            r2 = w.sep(q, r);
            const T bs = w.band(hsT);
            if (r2 > hsT * hsT + bs) continue;
            double rx2 = -1.0;
            if (!(r2 < hsT * hsT - bs)) {
                rx2 = exact_r2<D>(*st, xi, j, *pb);
                if (!(rx2 < hs2)) continue;
            }
            if (restricted) {
                const T bf = w.band(hfT);
                if (r2 > hfT * hfT + bf) continue;
                if (!(r2 < hfT * hfT - bf)) {
                    if (rx2 < 0.0) rx2 = exact_r2<D>(*st, xi, j, *pb);
                    if (!(__dsqrt_rn(rx2) < hf)) continue;
                }
            }
            return true;
        }
        return false;
    }

    template <class F>
    __device__ __forceinline__ void newton_pass(F f)
    {
        int stk[WALK_STACK];
        TargetWalk<D, T> w;
        w.start(stk, *tv, *pb, xi, root, hs, false);
        if (!active) w.sp = 0;
        T r[D], r2;
        V4 q;
        int j;
        while (next(w, r, r2, q, j)) f(sqrt(r2), q.w, T(0), T(0), false);
    }

    __device__ __forceinline__ void restrict(double h)
    {
        hf = h;
        restricted = true;
    }

    template <class F>
    __device__ __forceinline__ void for_members(bool load_v, F f)
    {
        int stk[WALK_STACK];
        TargetWalk<D, T> w;
        w.start(stk, *tv, *pb, xi, root, fmin(hs, hf), false);
        if (!active) w.sp = 0;
        T r[D], r2;
        V4 q;
        int j;
        while (next(w, r, r2, q, j)) {
            const V4 vj = load_v ? mvel[j] : V4{};
            f(r, r2, q.w, mu[j], j, vj);
        }
    }
};

// PreInteraction of target i (key slot) from its smoothing-length guess hg and search radius hs,
// over the pair source `src`:
//   newton_pass(f): f(r_a, m_a, r_b, m_b, two) for the candidates {j : r_ij < h_s} (one or two
//                   per call, r = |x_i - x_j| in T);
//   restrict(h):    the members from now on are the candidates with r_ij < h, decided exactly;
//   for_members(load_v, f): f(x_i - x_j in T, r^2, m_j, u_j, j, {v_j, c_j}) for each member
//                   ({v_j, c_j} loaded only when load_v).
// Warp-collective (the h / v_sig minimum and the Newton loop's exit test): all 32 lanes call it.
template <int D, typename T, int TYPE, int K, class Src>
__device__ __forceinline__ void pre_target(const PreArgs<T>& a, int i, int run, bool active, double hg, double hs,
                                           Src& src, int* iters_out, int* nnb_out)
{
    using V4 = typename Vec4<T>::type;
    using KF = Kern<D, K, T>;
    const State& st = a.st;
    const double mi = st.f[F_MASS][i];
        // ---- smoothing length: Newton-Raphson on rho h^D = b (or n h^D = b for disph) ----
        double h = hg;
        int iters = 0;
        if (!a.initial && a.iterative) {
            // N / A_D is a constant: one FP64 division per launch, not per target
            const T bconst = (T)((TYPE == 1) ? a.nn_over_a : mi * a.nn_over_a);
            bool done = !active, conv = false;
            for (int it = 0; it < 10; ++it) {
                if (!__any_sync(FULL, !done)) break;
                if (!done) {
                    ++iters;
                    const T hT = (T)h;
                    const T hinvT = T(1) / hT;
                    Sum<T> s0, s1;
                    s0.zero();
                    s1.zero();
                    // two candidates per call where the source pairs them: independent
                    // dependency chains, one compensated add per call
                    src.newton_pass([&](T rra, T ma, T rrb, T mb, bool two) {
                        T w = T(0), dw = T(0);
                        {
                            const T m = TYPE == 1 ? T(1) : ma;
                            const T W = KF::w(rra, hinvT), dW = KF::dhw(rra, hinvT);
                            if (rra < hT) { w = m * W; dw = m * dW; }
                        }
                        if (two) {
                            const T m = TYPE == 1 ? T(1) : mb;
                            const T W = KF::w(rrb, hinvT), dW = KF::dhw(rrb, hinvT);
                            if (rrb < hT) { w += m * W; dw += m * dW; }
                        }
                        s0.add(w);
                        s1.add(dw);
                    });
                    const T dens = (T)s0.get(), ddens = (T)s1.get();
                    const T hd = powD<D>(hT);
                    const T hd1 = D == 1 ? T(1) : D == 2 ? hT : hT * hT;
                    const T f = dens * hd - bconst;
                    const T df = ddens * hd + T(D) * dens * hd1;
                    const double hn = h - (double)(f / df);
                    if (fabs(hn - h) < (hn + h) * 1e-4) { done = true; conv = true; }
                    h = hn;
                }
            }
            if (active && !conv) {
                h = hg;   // PreInteraction::newton_raphson falls back to the unscaled guess
                atomicAdd(a.newton_fail, 1);
            }
        }
        const double hf = a.initial ? hg : (a.iterative ? h : hs);

        // ---- density, pressure, grad-h, signal velocity over {r < h} ----
        const T hT = (T)hf;
        const T hinvT = T(1) / hT;   // in the pair type (the FP64 divide costs 1/64-rate cycles)
        const T ciT = a.mvel[i].w;
        const T uiT = a.mu[i];
        T vi[3] = {T(0), T(0), T(0)};
        {
            const V4 v = a.mvel[i];
            vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
        }
        Sum<T> sd, sdh, sn, sp, sdp, sdn;
        sd.zero(); sdh.zero(); sn.zero(); sp.zero(); sdp.zero(); sdn.zero();
        // the Balsara / time-dependent-alpha sums over the same set {r < h}, accumulated in the
        // same pass (src/pre_interaction.cpp:115-161 normalise them only afterwards)
        const bool bal = a.use_balsara && D != 1;
        const bool avsum = TYPE != 2 && !a.initial && (bal || a.use_tdav);
        Sum<T> sdiv, srot[3];
        sdiv.zero(); srot[0].zero(); srot[1].zero(); srot[2].zero();
        T vsig = T(2) * ciT;
        int nnb = 0;
        {
            src.restrict(hf);
            src.for_members(!a.initial, [&](const T* r, T r2, T mj, T auxj, int j, const V4& vjr) {
                ++nnb;
                const T rr = sqrt(r2);
                const T W = KF::w(rr, hinvT);
                sd.add(mj * W);
                if (TYPE == 0) {
                    if (!a.initial) sdh.add(mj * KF::dhw(rr, hinvT));
                } else if (TYPE == 1) {
                    if (!a.initial) {
                        const T dW = KF::dhw(rr, hinvT);
                        const T muj = mj * auxj;
                        sn.add(W);
                        sp.add(muj * W);
                        sdp.add(muj * dW);
                        sdn.add(dW);
                    }
                }
                if (!a.initial && j != i) {
                    const V4 vj = vjr;
                    T vij[3] = {T(0), T(0), T(0)};
                    vij[0] = vi[0] - vj.x;
                    if (D > 1) vij[1] = vi[1] - vj.y;
                    if (D > 2) vij[2] = vi[2] - vj.z;
                    T rv = r[0] * vij[0];
                    if (D > 1) rv += r[D > 1 ? 1 : 0] * vij[1];
                    if (D > 2) rv += r[D > 2 ? 2 : 0] * vij[2];
                    const T vs = ciT + vj.w - T(3) * rv * (T(1) / rr);
                    vsig = vs > vsig ? vs : vsig;
                    if (avsum) {
                        // grad W = r_ij cf; the particle itself contributes dW = 0
                        const T cf = KF::dw_coef(rr, rr > T(0) ? T(1) / rr : T(0), hinvT);
                        const T wj = (TYPE == 1) ? mj * auxj : mj;
                        T dw[3] = {T(0), T(0), T(0)};
#pragma unroll
                        for (int k = 0; k < D; ++k) dw[k] = r[k] * cf;
                        T vd = vij[0] * dw[0];
                        if (D > 1) vd += vij[1] * dw[1];
                        if (D > 2) vd += vij[2] * dw[2];
                        sdiv.add(-wj * vd);
                        if (bal) {
                            if (D == 2) {
                                srot[0].add((vij[0] * dw[1] - vij[1] * dw[0]) * wj);
                            } else if (D == 3) {
                                srot[0].add((vij[1] * dw[2] - vij[2] * dw[1]) * wj);
                                srot[1].add((vij[2] * dw[0] - vij[0] * dw[2]) * wj);
                                srot[2].add((vij[0] * dw[1] - vij[1] * dw[0]) * wj);
                            }
                        }
                    }
                }
            });
        }
        *iters_out = iters;
        *nnb_out = nnb;
        if (a.initial) {
            if (active) {
                st.f[F_SML][i] = hf;
                st.f[F_DENS][i] = (double)sd.get();
            }
            return;
        }
        const double dens = (double)sd.get();
        const T densT = (T)dens;
        double pres;
        T gradh = T(0);
        if (TYPE == 0) {
            pres = (a.gamma - 1.0) * dens * (double)st.f[F_ENE][i];
            gradh = T(1) / (T(1) + hT / (T(D) * densT) * (T)sdh.get());
        } else if (TYPE == 1) {
            const T n_i = (T)sn.get();
            pres = (a.gamma - 1.0) * (double)sp.get();
            const T c = hT / (T(D) * n_i);
            gradh = c * (T)sdp.get() / (T(1) + c * (T)sdn.get());
        } else {
            pres = (a.gamma - 1.0) * dens * (double)st.f[F_ENE][i];
        }
        // h / v_sig minimum of the group -> run minimum (TimeStep input)
        {
            // minimum over the warp in T, converted once (the minimum commutes with the conversion)
            T hv = active ? hT / vsig : T(3.0e38f);
            for (int o = 16; o > 0; o >>= 1) { const T u = __shfl_xor_sync(FULL, hv, o); hv = u < hv ? u : hv; }
            if ((threadIdx.x & 31) == 0) atomicMin(&a.hvs[run], dbl_to_ord((double)hv));
        }

        if (TYPE == 2) {
            // ---- MUSCL gradients (src/gsph/g_pre_interaction.cpp:112-136) ----
            if (active) {
                st.f[F_SML][i] = hf;
                st.f[F_DENS][i] = dens;
                st.f[F_PRES][i] = pres;
                st.neighbor[i] = nnb;
            }
            if (!a.gsph_2nd) return;
            Sum<T> dd[D], du[D], dv[D][D];
#pragma unroll
            for (int k = 0; k < D; ++k) {
                dd[k].zero(); du[k].zero();
#pragma unroll
                for (int q = 0; q < D; ++q) dv[k][q].zero();
            }
            src.for_members(true, [&](const T* r, T r2, T mj, T auxj, int, const V4& vj) {
                    const T rr = sqrt(r2);
                    const T cf = KF::dw_coef(rr, rr > T(0) ? T(1) / rr : T(0), hinvT);
                    const T vjv[3] = {vj.x, vj.y, vj.z};
                    const T mdu = mj * (auxj - uiT);
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const T dw = r[k] * cf;
                        dd[k].add(dw * mj);
                        du[k].add(dw * mdu);
                    }
#pragma unroll
                    for (int q = 0; q < D; ++q) {
                        const T mv = mj * (vjv[q] - vi[q]);
#pragma unroll
                        for (int k = 0; k < D; ++k) dv[q][k].add(r[k] * cf * mv);
                    }
            });
            if (active) {
                const double ui = st.f[F_ENE][i];
                const T rho_inv = T(1) / densT;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const double ddk = (double)dd[k].get();
                    st.f[F_GRADD + k][i] = ddk;
                    st.f[F_GRADP + k][i] = (ddk * ui + (double)du[k].get()) * (a.gamma - 1.0);
                }
#pragma unroll
                for (int q = 0; q < D; ++q)
#pragma unroll
                    for (int k = 0; k < D; ++k) st.f[F_GRADV + q * 3 + k][i] = (double)((T)dv[q][k].get() * rho_inv);
            }
            return;
        }

        // ---- Balsara switch and time-dependent alpha (src/pre_interaction.cpp:115-161) ----
        T alpha = (T)st.f[F_ALPHA][i];
        T balsara = (T)st.f[F_BALSARA][i];
        double alpha_out = st.f[F_ALPHA][i], balsara_out = st.f[F_BALSARA][i];
        const T dt = (T)a.dt_run[run];
        if (avsum) {
            T div = (T)sdiv.get();
            T rot[3] = {(T)srot[0].get(), (T)srot[1].get(), (T)srot[2].get()};
            if (TYPE == 1) {
                const T p_inv = (T)(a.gamma - 1.0) / (T)pres;
                div *= p_inv;
                for (int k = 0; k < 3; ++k) rot[k] *= p_inv;
            } else {
                const T rho_inv = T(1) / densT;
                div *= rho_inv;
                for (int k = 0; k < 3; ++k) rot[k] *= rho_inv;
            }
            const T tau_inv = (T)a.eps_av * ciT / hT;
            if (bal) {
                const T rot_abs = D == 2 ? fabs(rot[0]) : sqrt(rot[0] * rot[0] + rot[1] * rot[1] + rot[2] * rot[2]);
                balsara = fabs(div) / (fabs(div) + rot_abs + T(1e-4) * ciT / hT);
                balsara_out = (double)balsara;
                if (a.use_tdav) {
                    const T sdv = -div > T(0) ? -div : T(0);
                    alpha_out = st.f[F_ALPHA][i] + (double)((-(alpha - (T)a.alpha_min) * tau_inv + sdv * ((T)a.alpha_max - alpha)) * dt);
                }
            } else {
                const T s_i = -div > T(0) ? -div : T(0);
                alpha_out = (double)((alpha + dt * tau_inv * (T)a.alpha_min + s_i * dt * (T)a.alpha_max) / (T(1) + dt * tau_inv + s_i * dt));
            }
        }
        if (active) {
            st.f[F_SML][i] = hf;
            st.f[F_DENS][i] = dens;
            st.f[F_PRES][i] = pres;
            st.f[F_GRADH][i] = (double)gradh;
            st.f[F_BALSARA][i] = balsara_out;
            st.f[F_ALPHA][i] = alpha_out;
            st.neighbor[i] = nnb;
            if (a.frec0) {
                // the records fluid_mirror_kernel forms, from the same doubles
                const double u = st.f[F_ENE][i], gh = (double)gradh;
                V4 r0, r1, r2;
                r0.x = vi[0];
                r0.y = D > 1 ? vi[D > 1 ? 1 : 0] : T(0);
                r0.z = D > 2 ? vi[D > 2 ? 2 : 0] : T(0);
                r1.x = (T)dens;
                r1.y = (T)pres;
                r1.z = ciT;
                r2.x = (T)alpha_out;
                r2.y = (T)balsara_out;
                r2.z = (T)u;
                if constexpr (std::is_same<T, float>::value) {
                    r0.w = __frcp_rn((float)hf);
                    r1.w = TYPE == 0 ? __fdiv_rn(__fdiv_rn(r1.y, r1.x), r1.x) * (float)gh : (float)gh;
                    r2.w = TYPE == 1 ? __fdiv_rn(r2.z, r1.y) : 0.0f;
                } else {
                    r0.w = (T)(1.0 / hf);
                    r1.w = TYPE == 0 ? (T)(pres / (dens * dens) * gh) : (T)gh;
                    r2.w = TYPE == 1 ? (T)(u / pres) : T(0);
                }
                a.frec0[i] = r0;
                a.frec1[i] = r1;
                a.frec2[i] = r2;
            }
        }
}

template <int D, typename T, int TYPE, int K>
__global__ void __launch_bounds__(256) pre_kernel(PreArgs<T> a)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    using V4 = typename Vec4<T>::type;
    using KF = Kern<D, K, T>;
    extern __shared__ __align__(16) unsigned char smem[];
    const SmemLayout L = a.L;
    GroupMisc* gm = reinterpret_cast<GroupMisc*>(smem + L.off_misc);
    const Tile<T> tile = tile_of<T>(smem, L);
    const State& st = a.st;
    const int t = threadIdx.x;
    const int GT = blockDim.x;
    constexpr double A = volume_const<D>();
    if (a.bulk_stage) bulk_stage_init(gm);

    for (;;) {
        int gb, gn;
        if (!next_group(gm, a.work, gb, gn)) break;
        if (gn == 0) continue;   // the unused half of an unsplit chunk
        // targets interleaved over the warps the group fills (warp w of nwa takes every nwa-th
        // target), so that they meet at the next group's barrier with similar amounts of work; the
        // CTA's other warps skip the group's pair work
        const int nwa = (gn + 31) >> 5;
        const bool warp_on = (t >> 5) < nwa;
        const int tl = warp_on ? (t & 31) * nwa + (t >> 5) : gn;
        const bool active = tl < gn;
        const int i = gb + (active ? tl : 0);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = st.f[F_POS + k][i];
        const double mi = st.f[F_MASS][i];
        // the guess (FP64 pow / sqrt) once per particle and stage: the group walk ahead of the
        // first pass, or else the first pass, stores it (for every target before any later pass)
        double hg;
        if (a.work.list == nullptr && a.pv.plan == nullptr) {
            hg = h_guess<D>((double)a.nn, mi, st.f[F_DENS][i]);
            if (active) a.hguess[i] = hg;
        } else {
            hg = a.hguess[i];
        }
        const double hs = a.initial ? hg : hg * a.ratio;
        const int run = st.run[gb];
        const int planned = load_plan<T>(smem, L, gm, a.pv);
        if (planned < 0) { report_overflow(a.work, gb, gn, gm); continue; }
        if (planned == 0) {
            group_box<D>(gm, xi, active, hs, a.pb);
            if (!group_walk<D, T>(smem, L, gm, a.tv, run, false, a.pb)) { report_overflow(a.work, gb, gn, gm); continue; }
        }
        {
            BoxAccept<D, T> box;
            box.init(gm);
            const T Rt = to_T_up<T>(gm->R);
            const T* mu = a.mu;
            const int ntile = stage_sources<D, T>(smem, L, gm, a.xrel, tile, [&](int, const T* off) {
                return box(off, Rt);
            }, [&](int j) { return mu[j]; }, a.bulk_stage != 0, a.work.err);
            if (ntile < 0) { report_overflow(a.work, gb, gn, gm); continue; }
            gm->ntile = ntile;   // every thread writes the same value
        }
        const int ntile = gm->ntile;
        const int nw = (ntile + 31) >> 5;
        T xo[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xo[k] = (T)min_image(xi[k] - gm->gc[k], a.pb, k);

        // ---- candidates: r^2 < h_s^2, exactly (src/bhtree.cpp:256) ----
        unsigned long long wmask = 0ull;   // words holding candidates (tiles of at most 64 words)
        int ncand = 0;
        {
            const double hs2 = __dmul_rn(hs, hs);
            const double band = r2_band<T, D>(gm, hs);
            const T lo_t = to_T_down<T>(hs2 - band), hi_t = to_T_up<T>(hs2 + band);
            for (int w = 0; w < nw; ++w) {
                unsigned bits = 0, band = 0;
                if (warp_on && word_box_r2<D, T>(xo, tile, w) <= hi_t) {   // else no source of the word is in
                    const int smax = min(32, ntile - w * 32);
                    unsigned inner = 0u;   // r2 <= hi_t
                    if (smax == 32) {
                        // a full word: unrolled, with constant bit positions and all its shared loads
                        // free to issue ahead
#pragma unroll
                        for (int b = 0; b < 32; ++b) {
                            T r[D];
                            const T r2 = tile_r2<D, T>(xo, tile.pm[w * 32 + b], r);
                            bits |= r2 < lo_t ? (1u << b) : 0u;
                            inner |= r2 <= hi_t ? (1u << b) : 0u;
                        }
                    } else {
                        for (int b = 0; b < smax; ++b) {
                            T r[D];
                            const T r2 = tile_r2<D, T>(xo, tile.pm[w * 32 + b], r);
                            bits |= r2 < lo_t ? (1u << b) : 0u;
                            inner |= r2 <= hi_t ? (1u << b) : 0u;
                        }
                    }
                    band = inner & ~bits;
                    // the guard band after the word, as a loop: a test inside the loop above is
                    // if-converted, which issues the FP64 re-decision for every source
                    while (band) {
                        const int b = __ffs(band) - 1;
                        band &= band - 1;
                        if (exact_r2<D>(st, xi, tile.idx[w * 32 + b], a.pb) < hs2) bits |= 1u << b;
                    }
                }
                if (!active) bits = 0u;
                tile.mask[w * GT + t] = bits;
                ncand += __popc(bits);
                if (bits && w < 64) wmask |= 1ull << w;
            }
        }

        // ---- the target's PreInteraction over its candidate bits ----
        TilePreSource<D, T> src{&tile, &st, &a.pb, a.mvel, xi, xo, GT, t, nw, wmask, gm};
        int iters = 0, nnb = 0;
        pre_target<D, T, TYPE, K>(a, i, run, active, hg, hs, src, &iters, &nnb);
        if (a.counters) {
            const bool cnt = active && !a.initial;
            warp_count(a.counters + PC_PRE_GROUPS, t == 0 ? 1ull : 0ull);
            warp_count(a.counters + PC_PRE_TARGETS, cnt ? 1ull : 0ull);
            warp_count(a.counters + PC_PRE_CANDIDATES, cnt ? (unsigned long long)ncand : 0ull);
            warp_count(a.counters + PC_PRE_ITERS, cnt ? (unsigned long long)iters : 0ull);
            warp_count(a.counters + PC_PRE_ITER_PAIRS, cnt ? (unsigned long long)iters * nnb : 0ull);
            warp_count(a.counters + PC_PRE_PAIRS, cnt ? (unsigned long long)nnb : 0ull);
            warp_count(a.counters + PC_PRE_TESTS, cnt ? (unsigned long long)ntile : 0ull);
        }
    }
}

// The thread-per-particle schedule of PreInteraction: a warp takes a target range (the group
// list, or the ranges an earlier group pass could not fit) and each lane one target, which walks
// the octree itself in each pass over its candidates.
template <int D, typename T, int TYPE, int K>
__global__ void __launch_bounds__(128) pre_tpp_kernel(PreArgs<T> a)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    const State& st = a.st;
    const int lane = threadIdx.x & 31;
    for (;;) {
        // a work item is one piece of 32 targets of a range, so that the few ranges a group pass
        // leaves spread over many warps instead of running one after another in one warp
        int k = 0;
        if (lane == 0) k = atomicAdd(a.work.counter, 1);
        k = __shfl_sync(FULL, k, 0);
        const int kr = k / a.work.pieces, o = 32 * (k % a.work.pieces);
        int gb = -1, gn = 0;
        if (a.work.list) {
            if (kr < min(*a.work.list_count, a.work.list_cap)) { const int2 r = a.work.list[kr]; gb = r.x; gn = r.y; }
        } else if (kr < *a.work.n_groups) {
            gb = a.work.g_begin[kr];
            gn = a.work.g_count[kr];
        }
        if (gb < 0) break;
        if (o < gn) {
            const bool active = o + lane < gn;
            const int i = gb + (active ? o + lane : 0);
            double xi[D];
#pragma unroll
            for (int q = 0; q < D; ++q) xi[q] = st.f[F_POS + q][i];
            double hg;
            if (a.work.list == nullptr) {
                hg = h_guess<D>((double)a.nn, st.f[F_MASS][i], st.f[F_DENS][i]);
                if (active) a.hguess[i] = hg;
            } else {
                hg = a.hguess[i];
            }
            const double hs = a.initial ? hg : hg * a.ratio;
            const int run = st.run[i];
            WalkPreSource<D, T> src{&a.tv, &a.pb, &st, a.xrel, a.mvel, a.mu, xi, hs, hs, run, active, false};
            int iters = 0, nnb = 0;
            pre_target<D, T, TYPE, K>(a, i, run, active, hg, hs, src, &iters, &nnb);
        }
    }
}

// The group plans of PreInteraction's first pass: per target the smoothing-length guess (stored
// for the pair passes) and the search radius h_s, then the group box and walk.
template <int D, typename T>
__global__ void __launch_bounds__(128) pre_walk_kernel(PreArgs<T> a, int stack_cap, int cap)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    extern __shared__ __align__(16) unsigned char smem[];
    const State& st = a.st;
    walk_groups<D, T>(a.work, a.tv, a.pb, st, false, a.pv, stack_cap, cap, [&](int i) {
        const double hg = h_guess<D>((double)a.nn, st.f[F_MASS][i], st.f[F_DENS][i]);
        a.hguess[i] = hg;
        return a.initial ? hg : hg * a.ratio;
    }, smem);
}

// Key-ordered T mirrors of the source fields Pre reads per pair.
template <int D, typename T>
__global__ void pre_mirror_kernel(State st, int n, typename Vec4<T>::type* mvel, T* mu, double c_sound)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double u = st.f[F_ENE][i];
    typename Vec4<T>::type v;
    v.x = (T)st.f[F_VEL][i];
    v.y = D > 1 ? (T)st.f[F_VEL + (D > 1 ? 1 : 0)][i] : T(0);
    v.z = D > 2 ? (T)st.f[F_VEL + (D > 2 ? 2 : 0)][i] : T(0);
    v.w = mirror_sound<T>(st, i, u, c_sound);
    mvel[i] = v;
    mu[i] = (T)u;
}

static __global__ void pre_reset_kernel(int R, long long* hvs, int* counters, int ncounters)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) hvs[r] = dbl_to_ord(1.7976931348623157e308);
    if (r < ncounters) counters[r] = 0;
}

}  // namespace sphgpu

// ---------------------------------------------------------------------------------------------
// Launcher (host).
namespace sphgpu {

template <int D>
constexpr int default_tile_cap() { return D == 1 ? 128 : D == 2 ? 512 : 1024; }

template <int D, typename T, int TYPE, int K>
void run_pre(Ctx& c, bool initial)
{
    using V4 = typename Vec4<T>::type;
    auto kern = pre_kernel<D, T, TYPE, K>;
    cudaStream_t s = c.stream;
    pre_mirror_kernel<D, T><<<ceil_div(c.n, 256), 256, 0, s>>>(c.st, c.n, (V4*)c.mir[0], (T*)c.mir[1],
                                                              c.sound_from_ene ? c.p.gamma * (c.p.gamma - 1.0) : 0.0);
    // counters: [0] main work, [1] overflow count, [2] overflow work; plus h/v_sig and Newton
    if (!initial) pre_reset_kernel<<<ceil_div(std::max(c.R, 48), 128), 128, 0, s>>>(c.R, c.d_hvs, c.d_work, 48);
    else pre_reset_kernel<<<1, 64, 0, s>>>(0, c.d_hvs, c.d_work, 48);
    cudaMemsetAsync(c.d_newton_fail, 0, sizeof(int), s);
    PreArgs<T> a{};
    a.st = c.st;
    a.tv = tree_view(c);
    a.pb = c.pb;
    a.xrel = (const V4*)c.mir[6];
    a.mvel = (const V4*)c.mir[0];
    a.mu = (const T*)c.mir[1];
    a.nn = c.p.neighbor_number;
    a.ratio = c.p.iterative_sml ? 1.2 : 1.0;
    a.gamma = c.p.gamma;
    a.iterative = c.p.iterative_sml;
    a.initial = initial ? 1 : 0;
    a.use_balsara = c.p.use_balsara;
    a.use_tdav = c.p.use_tdav;
    a.gsph_2nd = c.p.gsph_2nd_order;
    a.alpha_min = c.p.alpha_min;
    a.alpha_max = c.p.alpha_max;
    a.eps_av = c.p.epsilon_av;
    a.dt_run = c.d_dt;
    a.hvs = c.d_hvs;
    a.newton_fail = c.d_newton_fail;
    a.hguess = (double*)c.mir[8];
    a.nn_over_a = (double)c.p.neighbor_number / volume_const<D>();
    a.counters = c.count_work ? c.d_counters : nullptr;
    a.bulk_stage = c.bulk_stage;
    // inside a whole step the finished targets also write FluidForce's records (not gsph, whose
    // records come with its gradients), and FluidForce then skips its mirror kernel
    const bool frec = !initial && c.sound_from_ene && c.p.sph_type != 2;
    a.frec0 = frec ? (V4*)c.mir[2] : nullptr;
    a.frec1 = frec ? (V4*)c.mir[3] : nullptr;
    a.frec2 = frec ? (V4*)c.mir[4] : nullptr;
    c.fluid_records_fresh = frec;
    const int tcap = c.tile_cap_pre ? c.tile_cap_pre : default_tile_cap<D>();
    a.pv = PlanView<T>{};
    if ((c.prewalk & 2) && c.pair_sched != 3) {
        a.pv = plan_view<T>(c);
        const int cap = first_pass_leaf_cap(c), scap = std::max(128, cap);
        a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + PLAN_WORK_SLOT, nullptr, nullptr, 0,
                           nullptr, nullptr, 0, 0, c.d_err, nullptr};
        launch_plans((const void*)pre_walk_kernel<D, T>, c, plan_warp_bytes<T>(scap, cap),
                     [&](int grid, size_t smem) { pre_walk_kernel<D, T><<<grid, 128, smem, c.stream>>>(a, scap, cap); });
    }
    launch_pair_passes<PreArgs<T>>(c, (const void*)kern, a, tcap, sizeof(V4), sizeof(T),
        [](const void* k, int grid, int block, size_t smem, cudaStream_t st, PreArgs<T>& args) {
            reinterpret_cast<void (*)(PreArgs<T>)>(const_cast<void*>(k))<<<grid, block, smem, st>>>(args);
        },
        (const void*)pre_tpp_kernel<D, T, TYPE, K>,
        [](const void* k, int grid, int block, cudaStream_t st, PreArgs<T>& args) {
            reinterpret_cast<void (*)(PreArgs<T>)>(const_cast<void*>(k))<<<grid, block, 0, st>>>(args);
        });
}

}  // namespace sphgpu
