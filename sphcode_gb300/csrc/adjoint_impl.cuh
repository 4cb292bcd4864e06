// Reverse mode of one PreInteraction + FluidForce on the device, standard form (TYPE 0) or
// pressure-energy form (TYPE 1), and the leapfrog around it (Solver::predict / correct,
// src/solver.cpp:431-474).
//
// After the forward quantities of a step have been recomputed (prediction, tree, PreInteraction
// with its Newton smoothing lengths), five launches run the backward pass in key order:
//   prep    per particle: T mirrors of v, h, rho, P, c, grad-h, Balsara and of the adjoints of
//           a and du/dt that the force pass consumes (correct backward folded in);
//   pass 1  CTA per target group: the density-type sums the local backward needs (d rho/dh,
//           d2 rho/dh2, the div v / rot v sums and their h derivatives) and the fluid pair VJP
//           in both directions, i.e. the part of every pair term of a_t, du_t that depends on
//           this particle's inputs whether it is the target t or the source s
//           (adjoint_math.cuh: fluid_pair_vjp);
//   local   per particle: adjoints of rho, P, grad-h, h, c, Balsara to the weights of the
//           density-type sums, with the implicit smoothing length (pre_local_backward);
//   pass 2  CTA per target group: position and velocity gradients of those sums from both
//           members of every pair (pre_pair_gather);
//   final   per particle: predict backward, scatter to the caller's order, and the avAlpha
//           adjoint reduced per block (then one block sums the partials in a fixed order).
// Every particle gathers what it needs from its pair set {j : r_ij < max(h_i, h_j)}, so the
// passes are deterministic and need no atomics.  Pair terms are continuous at the edge of the
// kernel support, so the membership test needs no exact guard band: the mask keeps a slightly
// larger set and the terms outside the support evaluate to zero.
#pragma once

#include "adjoint_math.cuh"
#include "context.cuh"
#include "group.cuh"

namespace sphgpu {

template <typename T>
struct AdjArgs {
    using V4 = typename Vec4<T>::type;
    State st;
    TreeView tv;
    Periodic pb;
    SmemLayout L;
    GroupWork work;
    const V4* xrel;   // {x - leaf centre, m}
    const T* hmir;    // h
    const V4* a0;     // {v_0, v_1, v_2, h}
    const V4* a1;     // {rho, P, c, grad-h}
    const V4* a2;     // {Balsara, dubar, abar_0, abar_1}
    const V4* a3;     // {abar_2, u, 0, 0}
    const V4* w0;     // {w_rho, w_rhoh, Dbar, Rtbar_0}
    const V4* w1;     // {Rtbar_1, Rtbar_2, w_n, w_nh}
    const V4* w2;     // {w_Y, w_Yh, 0, 0}
    double* buf;
    int n;
    T alpha;
    T gamma;
};

// Walk and staging of the pair set of a target group; fills the per-target candidate masks and
// returns the number of mask words, or -1 when the group has to go to a later pass.
template <int D, typename T>
__device__ int adj_stage(unsigned char* smem, const AdjArgs<T>& a, GroupMisc* gm, const Tile<T>& tile,
                         int gb, bool active, const double* xi, double hi, T* xo)
{
    const SmemLayout& L = a.L;
    group_box<D>(gm, xi, active, hi, a.pb);
    const int run = a.st.run[gb];
    if (!group_walk<D, T>(smem, L, gm, a.tv, run, true, a.pb)) return -1;
    {
        BoxAccept<D, T> box;
        box.init(gm);
        const T Rt = to_T_up<T>(gm->R);
        const T* hmir = a.hmir;
        const int ntile = stage_sources<D, T>(smem, L, gm, a.xrel, tile, [&](int j, const T* off) {
            const T hj = hmir[j];
            return box(off, Rt > hj ? Rt : hj);
        }, [&](int j) { return hmir[j]; });
        if (ntile < 0) return -1;
        gm->ntile = ntile;
    }
    const int ntile = gm->ntile;
    const int nw = (ntile + 31) >> 5;
#pragma unroll
    for (int k = 0; k < D; ++k) xo[k] = (T)min_image(xi[k] - gm->gc[k], a.pb, k);
    const T h_i = (T)hi;
    const T grow = T(1.001);
    const int t = threadIdx.x, GT = blockDim.x;
    for (int w = 0; w < nw; ++w) {
        unsigned bits = 0;
        const T wmax = D == 3 ? tile.wbox[2 * w + 1].w : h_i;   // largest h_j of the word
        const T Hw = (h_i > wmax ? h_i : wmax) * grow;
        if (word_box_r2<D, T>(xo, tile, w) < Hw * Hw) {
            const int smax = min(32, ntile - w * 32);
            for (int b = 0; b < smax; ++b) {
                const int s = w * 32 + b;
                T r[D];
                const T r2 = tile_r2<D, T>(xo, tile.pm[s], r);
                const T hj = tile.aux[s];
                const T H = (h_i > hj ? h_i : hj) * grow;
                if (r2 < H * H) bits |= 1u << b;
            }
        }
        tile.mask[w * GT + t] = active ? bits : 0u;
    }
    return nw;
}

template <int D, typename T, int TYPE>
__device__ __forceinline__ sphadj::FluidSide<T> adj_side(const AdjArgs<T>& a, int j, T m, T h)
{
    using V4 = typename Vec4<T>::type;
    sphadj::FluidSide<T> s;
    const V4 q0 = a.a0[j], q1 = a.a1[j], q2 = a.a2[j];
    s.v[0] = q0.x; s.v[1] = q0.y; s.v[2] = q0.z;
    s.rho = q1.x; s.P = q1.y; s.c = q1.z; s.g = q1.w;
    s.B = q2.x; s.dubar = q2.y;
    s.abar[0] = q2.z; s.abar[1] = q2.w; s.abar[2] = T(0);
    s.u = T(0);
    if (D == 3 || TYPE == 1) {
        const V4 q3 = a.a3[j];
        if (D == 3) s.abar[2] = q3.x;
        s.u = q3.y;
    }
    s.h = h;
    s.m = m;
    return s;
}

template <int D, typename T, int TYPE>
__device__ __forceinline__ sphadj::PreWeights<T> adj_weights(const AdjArgs<T>& a, int j)
{
    using V4 = typename Vec4<T>::type;
    sphadj::PreWeights<T> w;
    const V4 p0 = a.w0[j];
    w.w_rho = p0.x; w.w_rhoh = p0.y; w.Dbar = p0.z;
    w.Rtbar[0] = p0.w; w.Rtbar[1] = T(0); w.Rtbar[2] = T(0);
    w.w_n = w.w_nh = w.w_Y = w.w_Yh = T(0);
    if (D == 3 || TYPE == 1) {
        const V4 p1 = a.w1[j];
        w.Rtbar[1] = p1.x; w.Rtbar[2] = p1.y;
        w.w_n = p1.z; w.w_nh = p1.w;
    }
    if (TYPE == 1) {
        const V4 p2 = a.w2[j];
        w.w_Y = p2.x; w.w_Yh = p2.y;
    }
    return w;
}

template <int D, typename T, int K, int TYPE>
__global__ void __launch_bounds__(256) adj_pass1_kernel(AdjArgs<T> a)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    extern __shared__ __align__(16) unsigned char smem[];
    const SmemLayout L = a.L;
    GroupMisc* gm = reinterpret_cast<GroupMisc*>(smem + L.off_misc);
    const Tile<T> tile = tile_of<T>(smem, L);
    const int t = threadIdx.x;
    const int GT = blockDim.x;
    const size_t n = (size_t)a.n;
    constexpr int NR = D == 3 ? 3 : D == 2 ? 1 : 0;   // components of the rot v sum

    for (;;) {
        int gb, gn;
        if (!next_group(gm, a.work, gb, gn)) break;
        if (gn == 0) continue;
        const bool active = t < gn;
        const int i = gb + (active ? t : 0);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = a.st.f[F_POS + k][i];
        const double hi = a.st.f[F_SML][i];
        T xo[D];
        const int nw = adj_stage<D, T>(smem, a, gm, tile, gb, active, xi, hi, xo);
        if (nw < 0) { report_overflow(a.work, gb, gn, gm); continue; }

        const T h_i = (T)hi;
        const T m_i = (T)a.st.f[F_MASS][i];
        const sphadj::FluidSide<T> si = adj_side<D, T, TYPE>(a, i, m_i, h_i);
        const T s_i = K == 0 ? T(0.5) * h_i : h_i;
        const T sinv_i = T(1) / s_i, hinv_i = T(1) / h_i;
        Sum<T> rho_h, rho_hh, dv, dv_h, rt[3], rt_h[3];
        Sum<T> xb[D], vb[D], rhob, pb, gb_, hb, cb, bb, ab;
        Sum<T> nd, nd_h, nd_hh, y_h, y_hh, ub;   // pressure-energy form
        rho_h.zero(); rho_hh.zero(); dv.zero(); dv_h.zero();
        nd.zero(); nd_h.zero(); nd_hh.zero(); y_h.zero(); y_hh.zero(); ub.zero();
#pragma unroll
        for (int k = 0; k < 3; ++k) { rt[k].zero(); rt_h[k].zero(); }
#pragma unroll
        for (int k = 0; k < D; ++k) { xb[k].zero(); vb[k].zero(); }
        rhob.zero(); pb.zero(); gb_.zero(); hb.zero(); cb.zero(); bb.zero(); ab.zero();

        MaskIter it(tile.mask, GT, t, nw);
        int s;
        while (it.next(s)) {
            T rv[3] = {T(0), T(0), T(0)};
            const T r2 = tile_r2<D, T>(xo, tile.pm[s], rv);
            const int j = tile.idx[s];
            const T h_j = tile.aux[s];
            const T m_j = tile.pm[s].w;
            const sphadj::FluidSide<T> sj = adj_side<D, T, TYPE>(a, j, m_j, h_j);
            T vij[3] = {T(0), T(0), T(0)};
#pragma unroll
            for (int k = 0; k < D; ++k) vij[k] = si.v[k] - sj.v[k];
            sphadj::PreSums<T> ps;
            ps.zero();
            sphadj::SideAdj<T> mine;
            mine.zero();
            T alpha_bar = T(0);
            if (r2 == T(0)) {
                // the particle itself (or one at the same position): only the density-type sums;
                // FluidForce skips r == 0
                sphadj::pre_sums_self<D, K, T, TYPE>(ps, m_j, sj.u, h_i);
            } else {
                sphadj::pass1_pair<D, K, T, TYPE>(rv, vij, r2, si, sj, s_i, sinv_i, hinv_i, T(1) / h_j, a.alpha,
                                                  a.gamma, ps, mine, alpha_bar);
            }
            rho_h.add(ps.rho_h);
            if (TYPE == 0) {
                rho_hh.add(ps.rho_hh);
            } else {
                nd.add(ps.n);
                nd_h.add(ps.n_h);
                nd_hh.add(ps.n_hh);
                y_h.add(ps.Y_h);
                y_hh.add(ps.Y_hh);
            }
            dv.add(ps.Dv);
            dv_h.add(ps.Dv_h);
#pragma unroll
            for (int k = 0; k < NR; ++k) { rt[k].add(ps.Rt[k]); rt_h[k].add(ps.Rt_h[k]); }
            if (r2 == T(0)) continue;
#pragma unroll
            for (int k = 0; k < D; ++k) { xb[k].add(mine.x[k]); vb[k].add(mine.v[k]); }
            rhob.add(mine.rho);
            pb.add(mine.P);
            gb_.add(mine.g);
            hb.add(mine.h);
            cb.add(mine.c);
            bb.add(mine.B);
            ab.add(alpha_bar);
            if (TYPE == 1) ub.add(mine.u);
        }
        if (active) {
            double* B = a.buf;
            B[AS_RHOH * n + i] = (double)rho_h.get();
            B[AS_RHOHH * n + i] = (double)rho_hh.get();
            B[AS_DV * n + i] = (double)dv.get();
            B[AS_DVH * n + i] = (double)dv_h.get();
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                B[(AS_RT + k) * n + i] = k < NR ? (double)rt[k].get() : 0.0;
                B[(AS_RTH + k) * n + i] = k < NR ? (double)rt_h[k].get() : 0.0;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                B[(AL_X + k) * n + i] = k < D ? (double)xb[k < D ? k : 0].get() : 0.0;
                B[(AL_V + k) * n + i] = k < D ? (double)vb[k < D ? k : 0].get() : 0.0;
            }
            B[AL_RHO * n + i] = (double)rhob.get();
            B[AL_P * n + i] = (double)pb.get();
            B[AL_G * n + i] = (double)gb_.get();
            B[AL_H * n + i] = (double)hb.get();
            B[AL_C * n + i] = (double)cb.get();
            B[AL_B * n + i] = (double)bb.get();
            B[AL_ALPHA * n + i] = (double)ab.get();
            if (TYPE == 1) {
                B[AS_N * n + i] = (double)nd.get();
                B[AS_NH * n + i] = (double)nd_h.get();
                B[AS_NHH * n + i] = (double)nd_hh.get();
                B[AS_YH * n + i] = (double)y_h.get();
                B[AS_YHH * n + i] = (double)y_hh.get();
                B[AL_U * n + i] = (double)ub.get();
            }
        }
    }
}

template <int D, typename T, int K, int TYPE>
__global__ void __launch_bounds__(256) adj_pass2_kernel(AdjArgs<T> a)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    using V4 = typename Vec4<T>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    const SmemLayout L = a.L;
    GroupMisc* gm = reinterpret_cast<GroupMisc*>(smem + L.off_misc);
    const Tile<T> tile = tile_of<T>(smem, L);
    const int t = threadIdx.x;
    const int GT = blockDim.x;
    const size_t n = (size_t)a.n;

    for (;;) {
        int gb, gn;
        if (!next_group(gm, a.work, gb, gn)) break;
        if (gn == 0) continue;
        const bool active = t < gn;
        const int i = gb + (active ? t : 0);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = a.st.f[F_POS + k][i];
        const double hi = a.st.f[F_SML][i];
        T xo[D];
        const int nw = adj_stage<D, T>(smem, a, gm, tile, gb, active, xi, hi, xo);
        if (nw < 0) { report_overflow(a.work, gb, gn, gm); continue; }

        const T h_i = (T)hi;
        const T m_i = (T)a.st.f[F_MASS][i];
        const T s_i = K == 0 ? T(0.5) * h_i : h_i;
        const T sinv_i = T(1) / s_i, hinv_i = T(1) / h_i;
        const V4 q0 = a.a0[i];
        const T v_i[3] = {q0.x, q0.y, q0.z};
        const T u_i = TYPE == 1 ? a.a3[i].y : T(0);
        const sphadj::PreWeights<T> wi = adj_weights<D, T, TYPE>(a, i);
        Sum<T> xb[D], vb[D], ub;
#pragma unroll
        for (int k = 0; k < D; ++k) { xb[k].zero(); vb[k].zero(); }
        ub.zero();

        MaskIter it(tile.mask, GT, t, nw);
        int s;
        while (it.next(s)) {
            T rv[3] = {T(0), T(0), T(0)};
            const T r2 = tile_r2<D, T>(xo, tile.pm[s], rv);
            const int j = tile.idx[s];
            if (j == i || r2 == T(0)) continue;
            const T h_j = tile.aux[s];
            const T m_j = tile.pm[s].w;
            const V4 p0 = a.a0[j];
            T vij[3] = {v_i[0] - p0.x, v_i[1] - p0.y, v_i[2] - p0.z};
            if (D < 3) vij[2] = T(0);
            if (D < 2) vij[1] = T(0);
            const sphadj::PreWeights<T> wj = adj_weights<D, T, TYPE>(a, j);
            T dx[3] = {T(0), T(0), T(0)}, dvv[3] = {T(0), T(0), T(0)};
            const T rinv = T(1) / sqrt(r2);
            const T r = r2 * rinv;
            const T hinv_j = T(1) / h_j;
            const T s_j = K == 0 ? T(0.5) * h_j : h_j;
            const T sinv_j = K == 0 ? T(2) * hinv_j : hinv_j;
            sphadj::KVals<T> ki, kj;
            sphadj::kvals<D, K, T, true>(r, rinv, s_i, sinv_i, hinv_i, ki);
            sphadj::kvals<D, K, T, true>(r, rinv, s_j, sinv_j, hinv_j, kj);
            if (TYPE == 0) {
                sphadj::pre_pair_gather_k<D, T>(rv, vij, rinv, m_j, ki, wi, dx, dvv);
                sphadj::pre_pair_gather_k<D, T>(rv, vij, rinv, m_i, kj, wj, dx, dvv);
            } else {
                // i's sums hold j (its u adjoint is j's), j's sums hold i
                T u_other = T(0), u_mine = T(0);
                const T u_j = a.a3[j].y;
                sphadj::pre_pair_gather_disph_k<D, T>(rv, vij, rinv, m_j, u_j, ki, wi, dx, dvv, u_other);
                sphadj::pre_pair_gather_disph_k<D, T>(rv, vij, rinv, m_i, u_i, kj, wj, dx, dvv, u_mine);
                ub.add(u_mine);
            }
#pragma unroll
            for (int k = 0; k < D; ++k) { xb[k].add(dx[k]); vb[k].add(dvv[k]); }
        }
        if (active) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                a.buf[(AG_X + k) * n + i] = k < D ? (double)xb[k < D ? k : 0].get() : 0.0;
                a.buf[(AG_V + k) * n + i] = k < D ? (double)vb[k < D ? k : 0].get() : 0.0;
            }
            a.buf[AG_U * n + i] = (double)ub.get();
        }
    }
}

// ---- per-particle kernels (FP64) ---------------------------------------------------------------

// Offsets of the blocks of the caller-order adjoint vector.
struct AdjLayout {
    size_t xb, vb, ub, ab, dub;
};
inline AdjLayout adj_layout(int n, int D)
{
    const size_t nd = (size_t)n * D;
    return AdjLayout{0, nd, 2 * nd, 2 * nd + n, 3 * nd + n};
}

template <int D, typename T>
__global__ void adj_prep_kernel(State st, int n, AdjLayout lay, const double* adj, const double* dt_run,
                                int initial, typename Vec4<T>::type* a0, typename Vec4<T>::type* a1,
                                typename Vec4<T>::type* a2, typename Vec4<T>::type* a3)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t q = (size_t)st.id[i];
    const double half_dt = 0.5 * dt_run[st.run[i]];
    typename Vec4<T>::type v;
    v.x = (T)st.f[F_VEL][i];
    v.y = D > 1 ? (T)st.f[F_VEL + (D > 1 ? 1 : 0)][i] : T(0);
    v.z = D > 2 ? (T)st.f[F_VEL + (D > 2 ? 2 : 0)][i] : T(0);
    v.w = (T)st.f[F_SML][i];
    a0[i] = v;
    v.x = (T)st.f[F_DENS][i];
    v.y = (T)st.f[F_PRES][i];
    v.z = (T)st.f[F_SOUND][i];
    v.w = (T)st.f[F_GRADH][i];
    a1[i] = v;
    // adjoints of a and du/dt at the force pass: those of the state plus correct()'s use of them
    double abar[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; ++k)
        abar[k] = adj[lay.ab + q * D + k] + (initial ? 0.0 : adj[lay.vb + q * D + k] * half_dt);
    const double dubar = adj[lay.dub + q] + (initial ? 0.0 : adj[lay.ub + q] * half_dt);
    v.x = (T)st.f[F_BALSARA][i];
    v.y = (T)dubar;
    v.z = (T)abar[0];
    v.w = (T)abar[1];
    a2[i] = v;
    v.x = (T)abar[2];
    v.y = (T)st.f[F_ENE][i];
    v.z = v.w = T(0);
    a3[i] = v;
}

template <int D, typename T, int K, int TYPE>
__global__ void adj_local_kernel(State st, int n, double gamma, int balsara, const double* dens_bar, double* buf,
                                 typename Vec4<T>::type* w0, typename Vec4<T>::type* w1,
                                 typename Vec4<T>::type* w2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    sphadj::PreSums<double> ps;
    ps.rho_h = buf[AS_RHOH * N + i];
    ps.rho_hh = buf[AS_RHOHH * N + i];
    ps.Dv = buf[AS_DV * N + i];
    ps.Dv_h = buf[AS_DVH * N + i];
#pragma unroll
    for (int k = 0; k < 3; ++k) { ps.Rt[k] = buf[(AS_RT + k) * N + i]; ps.Rt_h[k] = buf[(AS_RTH + k) * N + i]; }
    double rhobar = buf[AL_RHO * N + i];
    if (dens_bar) rhobar += dens_bar[st.id[i]];
    sphadj::PreWeights<double> W;
    double ub = 0.0;
    if (TYPE == 0) {
        sphadj::pre_local_backward<D, double>(st.f[F_DENS][i], st.f[F_SML][i], st.f[F_SOUND][i], st.f[F_ENE][i],
                                              gamma, balsara != 0, ps, rhobar, buf[AL_P * N + i], buf[AL_G * N + i],
                                              buf[AL_H * N + i], buf[AL_C * N + i], buf[AL_B * N + i], W, ub);
    } else {
        ps.n = buf[AS_N * N + i];
        ps.n_h = buf[AS_NH * N + i];
        ps.n_hh = buf[AS_NHH * N + i];
        ps.Y_h = buf[AS_YH * N + i];
        ps.Y_hh = buf[AS_YHH * N + i];
        ub = buf[AL_U * N + i];
        sphadj::pre_local_backward_disph<D, K, double>(
            st.f[F_DENS][i], st.f[F_SML][i], st.f[F_SOUND][i], st.f[F_ENE][i], st.f[F_PRES][i], st.f[F_MASS][i],
            gamma, balsara != 0, ps, rhobar, buf[AL_P * N + i], buf[AL_G * N + i], buf[AL_H * N + i],
            buf[AL_C * N + i], buf[AL_B * N + i], W, ub);
    }
    buf[AU_LOC * N + i] = ub;
    typename Vec4<T>::type v;
    v.x = (T)W.w_rho;
    v.y = (T)W.w_rhoh;
    v.z = (T)W.Dbar;
    v.w = (T)W.Rtbar[0];
    w0[i] = v;
    v.x = (T)W.Rtbar[1];
    v.y = (T)W.Rtbar[2];
    v.z = (T)W.w_n;
    v.w = (T)W.w_nh;
    w1[i] = v;
    v.x = (T)W.w_Y;
    v.y = (T)W.w_Yh;
    v.z = v.w = T(0);
    w2[i] = v;
}

// Leapfrog backward and scatter to the caller's order.  Step: x' = x + vp dt, v' = v + a dt,
// u' = u + du dt with vp = v + a dt/2, up = u + du dt/2 (predict), then v'' = vp + a' dt/2,
// u'' = up + du' dt/2 (correct).  Initialisation: the forces of the initial state only.
template <int D>
__global__ void adj_final_kernel(State st, int n, AdjLayout lay, double* adj, const double* dt_run, int initial,
                                 const double* buf, double* partials)
{
    __shared__ double red[256];
    const size_t N = (size_t)n;
    double my_alpha = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t q = (size_t)st.id[i];
        const double dt = dt_run[st.run[i]];
        my_alpha += buf[AL_ALPHA * N + i];
        const double u1b = buf[AU_LOC * N + i] + buf[AG_U * N + i];
        if (initial) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                adj[lay.xb + q * D + k] += buf[(AL_X + k) * N + i] + buf[(AG_X + k) * N + i];
                adj[lay.vb + q * D + k] += buf[(AL_V + k) * N + i] + buf[(AG_V + k) * N + i];
                adj[lay.ab + q * D + k] = 0.0;
            }
            adj[lay.ub + q] += u1b;
            adj[lay.dub + q] = 0.0;
            continue;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double x1b = adj[lay.xb + q * D + k] + buf[(AL_X + k) * N + i] + buf[(AG_X + k) * N + i];
            const double v1b = buf[(AL_V + k) * N + i] + buf[(AG_V + k) * N + i];
            const double vpb = adj[lay.vb + q * D + k] + x1b * dt;
            adj[lay.xb + q * D + k] = x1b;
            adj[lay.vb + q * D + k] = v1b + vpb;
            adj[lay.ab + q * D + k] = v1b * dt + vpb * (0.5 * dt);
        }
        const double upb = adj[lay.ub + q];
        adj[lay.ub + q] = u1b + upb;
        adj[lay.dub + q] = u1b * dt + upb * (0.5 * dt);
    }
    red[threadIdx.x] = my_alpha;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

static __global__ void adj_alpha_sum_kernel(const double* partials, int nparts, double* alpha_bar)
{
    __shared__ double red[1024];
    red[threadIdx.x] = threadIdx.x < nparts ? partials[threadIdx.x] : 0.0;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *alpha_bar += red[0];
}

// ---- launcher ----------------------------------------------------------------------------------

template <int D, typename T, int K, int TYPE>
void run_adjoint(Ctx& c, double* adj, const double* dens_bar, double* alpha_bar, bool initial)
{
    using V4 = typename Vec4<T>::type;
    cudaStream_t s = c.stream;
    const int n = c.n;
    V4* mir = reinterpret_cast<V4*>(c.adj_mir);
    V4 *a0 = mir, *a1 = mir + n, *a2 = mir + 2 * (size_t)n, *a3 = mir + 3 * (size_t)n;
    V4 *w0 = mir + 4 * (size_t)n, *w1 = mir + 5 * (size_t)n, *w2 = mir + 6 * (size_t)n;
    const AdjLayout lay = adj_layout(n, D);
    adj_prep_kernel<D, T><<<ceil_div(n, 256), 256, 0, s>>>(c.st, n, lay, adj, c.d_dt, initial ? 1 : 0, a0, a1, a2, a3);

    AdjArgs<T> a{};
    a.st = c.st;
    a.tv = tree_view(c);
    a.pb = c.pb;
    a.xrel = (const V4*)c.mir[6];
    a.hmir = (const T*)c.mir[7];
    a.a0 = a0; a.a1 = a1; a.a2 = a2; a.a3 = a3; a.w0 = w0; a.w1 = w1; a.w2 = w2;
    a.buf = c.adj_buf;
    a.n = n;
    a.alpha = (T)c.p.av_alpha;
    a.gamma = (T)c.p.gamma;
    const int tcap = c.tile_cap ? c.tile_cap : (D == 1 ? 128 : D == 2 ? 384 : 1024);
    auto launcher = [](const void* k, int grid, int block, size_t smem, cudaStream_t st, AdjArgs<T>& args) {
        reinterpret_cast<void (*)(AdjArgs<T>)>(const_cast<void*>(k))<<<grid, block, smem, st>>>(args);
    };
    reset_work_counters(c);
    launch_pair_passes<AdjArgs<T>>(c, (const void*)adj_pass1_kernel<D, T, K, TYPE>, a, tcap, sizeof(V4), sizeof(T),
                                   launcher);
    adj_local_kernel<D, T, K, TYPE><<<ceil_div(n, 256), 256, 0, s>>>(c.st, n, c.p.gamma, c.p.use_balsara && D > 1,
                                                                    dens_bar, c.adj_buf, w0, w1, w2);
    reset_work_counters(c);
    launch_pair_passes<AdjArgs<T>>(c, (const void*)adj_pass2_kernel<D, T, K, TYPE>, a, tcap, sizeof(V4), sizeof(T),
                                   launcher);
    const int grid = std::min(ADJ_PARTIALS, ceil_div(n, 256));
    adj_final_kernel<D><<<grid, 256, 0, s>>>(c.st, n, lay, adj, c.d_dt, initial ? 1 : 0, c.adj_buf, c.adj_partials);
    adj_alpha_sum_kernel<<<1, 1024, 0, s>>>(c.adj_partials, grid, alpha_bar);
}

template <int D>
void adjoint_dispatch(Ctx& c, double* adj, const double* dens_bar, double* alpha_bar, bool initial)
{
    const bool f32 = c.precision == SPHGPU_FP32_PAIR;
    const int k = c.p.kernel, ty = c.p.sph_type;
#define SPHGPU_ADJ(T, K, TY) run_adjoint<D, T, K, TY>(c, adj, dens_bar, alpha_bar, initial)
    if (f32) {
        if (k == 0) { if (ty == 0) SPHGPU_ADJ(float, 0, 0); else SPHGPU_ADJ(float, 0, 1); }
        else { if (ty == 0) SPHGPU_ADJ(float, 1, 0); else SPHGPU_ADJ(float, 1, 1); }
    } else {
        if (k == 0) { if (ty == 0) SPHGPU_ADJ(double, 0, 0); else SPHGPU_ADJ(double, 0, 1); }
        else { if (ty == 0) SPHGPU_ADJ(double, 1, 0); else SPHGPU_ADJ(double, 1, 1); }
    }
#undef SPHGPU_ADJ
}

}  // namespace sphgpu
