// FluidForce on the device: pressure-gradient, artificial-viscosity and artificial-conductivity
// pair sums of the standard SPH form (src/fluid_force.cpp:26-116), of the pressure-energy form
// (src/disph/d_fluid_force.cpp:26-86) and of the Godunov form with MUSCL reconstruction and the
// HLL solver (src/gsph/g_fluid_force.cpp:28-199).
//
// One CTA per target group (group.cuh).  The pair set of target i is the reference's
// {j : r_ij < max(h_i, h_j), r_ij != 0}: the octree walk keeps leaves within max(R, node kernel
// size) of the group box (BHTree::neighbor_search with is_ij, src/bhtree.cpp:237), staging keeps
// sources within max(R, h_j) per axis, and the membership test runs in the pair type T outside a
// relative guard band and in the reference's FP64 arithmetic inside it.  Per-source fields are
// read from key-ordered mirror records in T.
#pragma once

#include "context.cuh"
#include "group.cuh"

namespace sphgpu {

// Per-particle gradient record of the second-order Godunov form (T): d rho/dx_k at d(k), dP/dx_k
// at p(k), dv_k/dx_d at v(k, d), padded to a multiple of four entries (1D: 4, 2D: 8, 3D: 16).
template <int D>
struct GradLayout {
    static constexpr int stride = D == 1 ? 4 : D == 2 ? 8 : 16;
    __host__ __device__ static constexpr int d(int k) { return k; }
    __host__ __device__ static constexpr int p(int k) { return D + k; }
    __host__ __device__ static constexpr int v(int k, int dd) { return 2 * D + D * k + dd; }
};

template <typename T>
struct FluidArgs {
    using V4 = typename Vec4<T>::type;
    State st;
    TreeView tv;
    Periodic pb;
    SmemLayout L;
    GroupWork work;
    const V4* xrel;   // {x - leaf centre, m}
    const T* hmir;    // h
    const V4* rec0;   // {vx, vy, vz, 1/h}
    const V4* rec1;   // {rho, P, c, X}   X: ssph P/rho^2 gradh, disph gradh, gsph 0
    const V4* rec2;   // {alpha, balsara, u, Y}   Y: disph u/P
    const T* grad;    // gsph: 16 per particle, grad rho [0,D), grad P [3,3+D), grad v [6 + 3k + d]
    double gamma;
    T gamma_t, gm1_t, alpha_ac_t;   // the same constants in T (formed on the host, no conversions per target)
    int use_ac;
    int ac_gravity;
    double alpha_ac;
    int gsph_2nd;
    const double* dt_run;
    unsigned long long* counters;   // PairCounter slots, or nullptr (not counted)
    int bulk_stage;                 // stage the tile with bulk asynchronous copies (knob 29)
    PlanView<T> pv;                 // group plans of the first pass (pv.plan nullptr: none)
};

// van Leer limiter (src/gsph/g_fluid_force.cpp:28-36).
template <typename T>
__device__ __forceinline__ T van_leer(T dq1, T dq2)
{
    const T p = dq1 * dq2;
    return p <= T(0) ? T(0) : T(2) * p / (dq1 + dq2);
}

// HLL Riemann solver with Roe-averaged wave speeds (src/gsph/g_fluid_force.cpp:168-199).
// left/right = {u, rho, p, c}.
template <typename T>
__device__ __forceinline__ void hll(const T* l, const T* r, T& pstar, T& vstar)
{
    const T roe_l = sqrt(l[1]), roe_r = sqrt(r[1]);
    const T roe_inv = T(1) / (roe_l + roe_r);
    const T u_t = (roe_l * l[0] + roe_r * r[0]) * roe_inv;
    const T c_t = (roe_l * l[3] + roe_r * r[3]) * roe_inv;
    const T s_l = fmin(l[0] - l[3], u_t - c_t);
    const T s_r = fmax(r[0] + r[3], u_t + c_t);
    const T c1 = l[1] * (s_l - l[0]);
    const T c2 = r[1] * (s_r - r[0]);
    const T c3 = T(1) / (c1 - c2);
    const T c4 = l[2] - l[0] * c1;
    const T c5 = r[2] - r[0] * c2;
    vstar = (c5 - c4) * c3;
    pstar = (c1 * c5 - c2 * c4) * c3;
}

// FluidForce of target i (key slot) over the pair source `src`, whose next() yields each member
// j of the target's pair set {j : r_ij < max(h_i, h_j), r_ij != 0} once, in a fixed order, with
// the separation x_i - x_j in T, r^2, m_j and 1/h_j.  Writes acc and du/dt of i when active.
template <int D, typename T, int TYPE, int K, class Src>
__device__ __forceinline__ void fluid_target(const FluidArgs<T>& a, int i, int run, bool active, Src& src)
{
    using V4 = typename Vec4<T>::type;
    using KF = Kern<D, K, T>;
    const State& st = a.st;
    const V4 r0i = a.rec0[i], r1i = a.rec1[i], r2i = a.rec2[i];
    const T vi[3] = {r0i.x, r0i.y, r0i.z};
    const T hinv_i = r0i.w;
        const T rho_i = r1i.x, p_i = r1i.y, c_i = r1i.z, X_i = r1i.w;
        const T al_i = r2i.x, b_i = r2i.y, u_i = r2i.z;
        const T m_i = a.xrel[i].w;   // the mass in T, as the sources carry it
        const T gm1 = a.gm1_t;
        // ssph: P_i/rho_i^2 gradh_i ; disph: (gamma-1)^2 u_i / P_i, (gamma-1)^2 u_i, 1/(m_i u_i)
        const T g2u_i = gm1 * gm1 * u_i;
        const T g2u_per_p_i = g2u_i / p_i;
        const T mu_inv_i = T(1) / (m_i * u_i);
        const T rho2_inv_i = T(1) / (rho_i * rho_i);
        const T dt = (T)a.dt_run[run];
        const T gamma = a.gamma_t;
        const T alpha_ac = a.alpha_ac_t;
        T gi[GradLayout<D>::stride];
        if (TYPE == 2 && a.gsph_2nd) {
#pragma unroll
            for (int q = 0; q < GradLayout<D>::stride; ++q) gi[q] = a.grad[(size_t)i * GradLayout<D>::stride + q];
        }

        Sum<T> acc[D], dene;
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k].zero();
        dene.zero();

        T rv[D], r2, mj, hinv_j;
        int j;
        while (src.next(rv, r2, mj, hinv_j, j)) {
            {
                const V4 r0j = a.rec0[j];
                const T rinv = rsqrt_t(r2);
                const T r = r2 * rinv;
                const T cfi = KF::dw_coef(r, rinv, hinv_i);
                const T cfj = KF::dw_coef(r, rinv, hinv_j);
                const V4 r1j = a.rec1[j];
                if (TYPE == 2) {
                    // ---- Godunov SPH pair (src/gsph/g_fluid_force.cpp:79-163) ----
                    const T rho_j = r1j.x, p_j = r1j.y, c_j = r1j.z;
                    const T r_inv = rinv;
                    T e[D];
#pragma unroll
                    for (int k = 0; k < D; ++k) e[k] = rv[k] * r_inv;
                    const T vj[3] = {r0j.x, r0j.y, r0j.z};
                    T ve_i = T(0), ve_j = T(0);
#pragma unroll
                    for (int k = 0; k < D; ++k) { ve_i += vi[k] * e[k]; ve_j += vj[k] * e[k]; }
                    T left[4], right[4];
                    if (a.gsph_2nd) {
                        const T* gj = a.grad + (size_t)j * GradLayout<D>::stride;
                        const T delta_i = T(0.5) * (T(1) - c_i * dt * r_inv);
                        const T delta_j = T(0.5) * (T(1) - c_j * dt * r_inv);
                        // velocity: e . (grad v) . e * r
                        T dve_i = T(0), dve_j = T(0);
#pragma unroll
                        for (int k = 0; k < D; ++k) {
                            T si = T(0), sj = T(0);
#pragma unroll
                            for (int d = 0; d < D; ++d) {
                                si += gi[GradLayout<D>::v(k, d)] * e[d];
                                sj += gj[GradLayout<D>::v(k, d)] * e[d];
                            }
                            dve_i += si * e[k];
                            dve_j += sj * e[k];
                        }
                        dve_i *= r;
                        dve_j *= r;
                        const T dv_ij = ve_i - ve_j;
                        right[0] = ve_i - van_leer(dv_ij, dve_i) * delta_i;
                        left[0] = ve_j + van_leer(dv_ij, dve_j) * delta_j;
                        T ddi = T(0), ddj = T(0), dpi = T(0), dpj = T(0);
#pragma unroll
                        for (int k = 0; k < D; ++k) {
                            ddi += gi[GradLayout<D>::d(k)] * e[k]; ddj += gj[GradLayout<D>::d(k)] * e[k];
                            dpi += gi[GradLayout<D>::p(k)] * e[k]; dpj += gj[GradLayout<D>::p(k)] * e[k];
                        }
                        ddi *= r; ddj *= r; dpi *= r; dpj *= r;
                        const T dd_ij = rho_i - rho_j, dp_ij = p_i - p_j;
                        right[1] = rho_i - van_leer(dd_ij, ddi) * delta_i;
                        left[1] = rho_j + van_leer(dd_ij, ddj) * delta_j;
                        right[2] = p_i - van_leer(dp_ij, dpi) * delta_i;
                        left[2] = p_j + van_leer(dp_ij, dpj) * delta_j;
                        right[3] = sqrt(gamma * right[2] / right[1]);
                        left[3] = sqrt(gamma * left[2] / left[1]);
                    } else {
                        right[0] = ve_i; right[1] = rho_i; right[2] = p_i; right[3] = c_i;
                        left[0] = ve_j; left[1] = rho_j; left[2] = p_j; left[3] = c_j;
                    }
                    T pstar, vstar;
                    hll<T>(left, right, pstar, vstar);
                    const T ci_ = mj * pstar * rho2_inv_i * cfi + mj * pstar / (rho_j * rho_j) * cfj;
                    // f = r_ij * ci_ ; dene -= f . (e vstar - v_i)
                    T fv = T(0);
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const T f = rv[k] * ci_;
                        acc[k].add(-f);
                        fv += f * (e[k] * vstar - vi[k]);
                    }
                    dene.add(-fv);
                } else {
                    const V4 r2j = a.rec2[j];
                    const T rho_j = r1j.x, p_j = r1j.y, c_j = r1j.z, X_j = r1j.w;
                    T vr = T(0);
                    vr += rv[0] * (vi[0] - r0j.x);
                    if (D > 1) vr += rv[D > 1 ? 1 : 0] * (vi[1] - r0j.y);
                    if (D > 2) vr += rv[D > 2 ? 2 : 0] * (vi[2] - r0j.z);
                    // Monaghan (1997) signal-velocity viscosity (src/fluid_force.cpp:89-106)
                    T pi_ij = T(0);
                    if (vr < T(0)) {
                        const T alpha = T(0.5) * (al_i + r2j.x);
                        const T bal = T(0.5) * (b_i + r2j.y);
                        const T w = vr * rinv;
                        const T vsig = c_i + c_j - T(3) * w;
                        const T rho_ij_inv = T(2) / (rho_i + rho_j);
                        pi_ij = T(-0.5) * bal * alpha * vsig * w * rho_ij_inv;
                    }
                    const T cfij = T(0.5) * (cfi + cfj);
                    T ac = T(0);
                    if (a.use_ac) {
                        // Wadsley et al. (2008) / Price (2008) (src/fluid_force.cpp:108-116)
                        const T vs = a.ac_gravity ? fabs(vr * rinv) : sqrt(T(2) * fabs(p_i - p_j) / (rho_i + rho_j));
                        ac = alpha_ac * mj * vs * (u_i - r2j.z) * (cfij * r);
                    }
                    T ai, aj, de_p;
                    if (TYPE == 0) {
                        ai = mj * (X_i + T(0.5) * pi_ij);
                        aj = mj * (X_j + T(0.5) * pi_ij);
                        de_p = mj * X_i * cfi * vr;
                    } else {
                        const T u_j = r2j.z;
                        const T f_ij = T(1) - X_i / (mj * u_j);
                        const T f_ji = T(1) - X_j * mu_inv_i;
                        const T t_i = g2u_per_p_i * u_j * f_ij;
                        ai = mj * (t_i + T(0.5) * pi_ij);
                        aj = mj * (g2u_i * r2j.w * f_ji + T(0.5) * pi_ij);
                        de_p = mj * t_i * cfi * vr;
                    }
                    const T cacc = cfi * ai + cfj * aj;
#pragma unroll
                    for (int k = 0; k < D; ++k) acc[k].add(-rv[k] * cacc);
                    dene.add(de_p + T(0.5) * mj * pi_ij * cfij * vr + ac);
                }
            }
        }
        if (active) {
#pragma unroll
            for (int k = 0; k < D; ++k) st.f[F_ACC + k][i] = (double)acc[k].get();
            st.f[F_DENE][i] = (double)dene.get();
        }
}

// Pair source of the group schedule: the candidate bits of target i over the CTA's staged tile,
// each decided exactly (T test outside the guard band, the reference's FP64 test inside it).
template <int D, typename T, class It>
struct TileSource {
    using V4 = typename Vec4<T>::type;
    It it;
    const Tile<T>* tile;
    const State* st;
    const Periodic* pb;
    const double* xi;
    const T* xo;
    double hi;
    T hinv_i, dlo;
    int i;
    __device__ __forceinline__ bool next(T* rv, T& r2, T& mj, T& hinv_j, int& j)
    {
        int s;
        while (it.next(s)) {
            const V4 p = tile->pm[s];
            r2 = tile_r2<D, T>(xo, p, rv);
            j = tile->idx[s];
            if (j == i) continue;
            hinv_j = tile->aux[s];
            const T Hinv = hinv_i < hinv_j ? hinv_i : hinv_j;
            if (!(r2 * (Hinv * Hinv) < dlo) || r2 == T(0)) {
                const double r2x = exact_r2<D>(*st, xi, j, *pb);
                const double rx = __dsqrt_rn(r2x);
                if (rx >= fmax(hi, st->f[F_SML][j]) || rx == 0.0) continue;
                if (r2 == T(0)) continue;   // unresolvable in T (coincident offsets)
            }
            mj = p.w;
            return true;
        }
        return false;
    }
};

// Pair source of the thread-per-particle schedule: the target's own walk (is_ij reach, the
// reference's BHTree::neighbor_search with is_ij) over the particles of the leaves it reaches,
// each decided exactly like the tile source's.
template <int D, typename T>
struct WalkSource {
    using V4 = typename Vec4<T>::type;
    TargetWalk<D, T> w;
    const V4* xrel;
    const V4* rec0;
    const T* hmir;
    const State* st;
    const Periodic* pb;
    double hi;
    T hiT;
    int i;
    __device__ __forceinline__ bool next(T* rv, T& r2, T& mj, T& hinv_j, int& j)
    {
        int jj;
        while (w.next(jj)) {
            if (jj == i) continue;
            const V4 q = xrel[jj];
            r2 = w.sep(q, rv);
            const T hj = hmir[jj];
            const T H = hiT > hj ? hiT : hj;
            const T band = w.band(H);
            if (!(r2 < H * H - band) || r2 == T(0)) {
                if (r2 > H * H + band) continue;
                const double r2x = exact_r2<D>(*st, w.xi, jj, *pb);
                const double rx = __dsqrt_rn(r2x);
                if (rx >= fmax(hi, st->f[F_SML][jj]) || rx == 0.0) continue;
                if (r2 == T(0)) continue;
            }
            j = jj;
            mj = q.w;
            hinv_j = rec0[jj].w;
            return true;
        }
        return false;
    }
};

template <int D, typename T, int TYPE, int K>
__global__ void __launch_bounds__(256) fluid_kernel(FluidArgs<T> a)
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
        const double hi = st.f[F_SML][i];
        const int run = st.run[gb];
        const int planned = load_plan<T>(smem, L, gm, a.pv);
        if (planned < 0) { report_overflow(a.work, gb, gn, gm); continue; }
        if (planned == 0) {
            group_box<D>(gm, xi, active, hi, a.pb);
            if (!group_walk<D, T>(smem, L, gm, a.tv, run, true, a.pb)) { report_overflow(a.work, gb, gn, gm); continue; }
        }
        // Relative guard band of the T-precision test r^2 < H^2 for H = max(h_i, h_j) >= h_min
        // of the group: the component error E (comp_err) at separations ~H is below e_rel H, so
        // |r2_T - r2| < delta H^2 there.  Group-uniform: formed by thread 0 (its FP64 arithmetic
        // once per group, not per target) and read after the staging's barriers.
        // (in the FP32 form formed in FP32 and widened by 0.1 %: a wider band only sends more
        // pairs to the exact test)
        if (threadIdx.x == 0) {
            const T hm = (T)gm->rmin;
            const T e_rel = (T)comp_err<T>(gm, gm->rmin) / hm * T(1.001) + (T)(Unit<T>::u * 3.0);
            const T dl = T(2.002) * (T(2.0 * 1.7320508075688772) * e_rel + T(D) * e_rel * e_rel + (T)(8.0 * Unit<T>::u));
            gm->bandf = (float)dl;
            gm->bandd = (double)dl;
        }
        {
            // keep sources within max(R, h_j) of the group box
            BoxAccept<D, T> box;
            box.init(gm);
            const T Rt = to_T_up<T>(gm->R);
            const T* hmir = a.hmir;
            const int ntile = stage_sources<D, T>(smem, L, gm, a.xrel, tile, [&](int j, const T* off) {
                const T hj = hmir[j];
                return box(off, Rt > hj ? Rt : hj);
            }, [&](int j) { return a.rec0[j].w; }, a.bulk_stage != 0, a.work.err);
            if (ntile < 0) { report_overflow(a.work, gb, gn, gm); continue; }
            gm->ntile = ntile;
        }
        const int ntile = gm->ntile;
        const int nw = (ntile + 31) >> 5;

        const T delta = sizeof(T) == 4 ? (T)gm->bandf : (T)gm->bandd;
        const T dlo = T(1) - delta, dhi = T(1) + delta;

        T xo[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xo[k] = (T)min_image(xi[k] - gm->gc[k], a.pb, k);
        const T hinv_i = a.rec0[i].w;

        // ---- pair candidates: r^2 < max(h_i, h_j)^2 (1 + delta), j != i ----
        unsigned long long wmask = 0ull;   // words holding candidates (tiles of at most 64 words)
        for (int w = 0; w < nw; ++w) {
            unsigned bits = 0;
            // the word's smallest 1/h_j bounds every source's 1/max(h_i, h_j) from below
            const T wmin = D == 3 ? tile.wbox[2 * w].w : hinv_i;
            const T Hw = hinv_i < wmin ? hinv_i : wmin;
            if (warp_on && word_box_r2<D, T>(xo, tile, w) * (Hw * Hw) < dhi) {
                const int smax = min(32, ntile - w * 32);
                auto test = [&](int b) -> unsigned {
                    const int s = w * 32 + b;
                    T r[D];
                    const T r2 = tile_r2<D, T>(xo, tile.pm[s], r);
                    const T hinv_j = tile.aux[s];
                    const T Hinv = hinv_i < hinv_j ? hinv_i : hinv_j;   // 1 / max(h_i, h_j)
                    return r2 * (Hinv * Hinv) < dhi ? (1u << b) : 0u;
                };
                if (smax == 32) {
                    // a full word: unrolled, with constant bit positions
#pragma unroll
                    for (int b = 0; b < 32; ++b) bits |= test(b);
                } else {
                    for (int b = 0; b < smax; ++b) bits |= test(b);
                }
            }
            if (!active) bits = 0u;
            tile.mask[w * GT + t] = bits;
            if (bits && w < 64) wmask |= 1ull << w;
        }

        // 3D tiles hold many words without candidates for a target; in 2D the plain scan is cheaper
        using It = typename std::conditional<D == 3, MaskWordIter, MaskIter>::type;
        TileSource<D, T, It> src{It(tile.mask, GT, t, nw, wmask), &tile, &st, &a.pb, xi, xo, hi, hinv_i, dlo, i};
        fluid_target<D, T, TYPE, K>(a, i, run, active, src);
        if (a.counters) {
            warp_count(a.counters + PC_FLUID_GROUPS, t == 0 ? 1ull : 0ull);
            warp_count(a.counters + PC_FLUID_TESTS, active ? (unsigned long long)ntile : 0ull);
        }
    }
}

// The group plans of FluidForce's first pass (search radius h_i, walk with node kernel sizes).
template <int D, typename T>
__global__ void __launch_bounds__(128) fluid_walk_kernel(FluidArgs<T> a, int stack_cap, int cap)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    extern __shared__ __align__(16) unsigned char smem[];
    const State& st = a.st;
    walk_groups<D, T>(a.work, a.tv, a.pb, st, true, a.pv, stack_cap, cap, [&](int i) { return st.f[F_SML][i]; }, smem);
}

// The thread-per-particle schedule: a warp takes a target range (the group list, or the ranges
// an earlier group pass could not fit) and each lane one target, which walks the octree itself
// and sums its pairs straight from the per-particle mirrors (no shared staging, no capacity but
// the walk stack's).
template <int D, typename T, int TYPE, int K>
__global__ void __launch_bounds__(128) fluid_tpp_kernel(FluidArgs<T> a)
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
            const double hi = st.f[F_SML][i];
            const int run = st.run[i];
            int stk[WALK_STACK];
            WalkSource<D, T> src;
            src.w.start(stk, a.tv, a.pb, xi, run, hi, true);
            if (!active) src.w.sp = 0;
            src.xrel = a.xrel;
            src.rec0 = a.rec0;
            src.hmir = a.hmir;
            src.st = &st;
            src.pb = &a.pb;
            src.hi = hi;
            src.hiT = (T)hi;
            src.i = i;
            fluid_target<D, T, TYPE, K>(a, i, run, active, src);
            if (src.w.overflow) atomicOr(a.work.err, (unsigned)ERR_STACK);
        }
    }
}

// Key-ordered T mirrors of the per-source fields of the force loop.
template <int D, typename T, int TYPE>
__global__ void fluid_mirror_kernel(State st, int n, typename Vec4<T>::type* rec0,
                                    typename Vec4<T>::type* rec1, typename Vec4<T>::type* rec2,
                                    T* grad, int gsph_2nd, double c_sound)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    typename Vec4<T>::type v;
    v.x = (T)st.f[F_VEL][i];
    v.y = D > 1 ? (T)st.f[F_VEL + (D > 1 ? 1 : 0)][i] : T(0);
    v.z = D > 2 ? (T)st.f[F_VEL + (D > 2 ? 2 : 0)][i] : T(0);
    const double rho = st.f[F_DENS][i], p = st.f[F_PRES][i];
    typename Vec4<T>::type b;
    b.x = (T)rho;
    b.y = (T)p;
    b.z = mirror_sound<T>(st, i, st.f[F_ENE][i], c_sound);
    typename Vec4<T>::type c;
    c.x = (T)st.f[F_ALPHA][i];
    c.y = (T)st.f[F_BALSARA][i];
    c.z = (T)st.f[F_ENE][i];
    if constexpr (std::is_same<T, float>::value) {
        // FP32 records: the quotients in FP32 (IEEE reciprocal and division) from the rounded
        // operands; FP64 divisions run at 1/64 of the FP32 rate and bound this kernel otherwise.
        // 1/h is within one FP32 ulp of 1/h_j, inside the membership test's guard band.
        v.w = __frcp_rn((float)st.f[F_SML][i]);
        b.w = TYPE == 0 ? __fdiv_rn(__fdiv_rn(b.y, b.x), b.x) * (float)st.f[F_GRADH][i]
            : TYPE == 1 ? (float)st.f[F_GRADH][i] : 0.0f;
        c.w = TYPE == 1 ? __fdiv_rn(c.z, b.y) : 0.0f;
    } else {
        v.w = (T)(1.0 / st.f[F_SML][i]);
        b.w = TYPE == 0 ? (T)(p / (rho * rho) * st.f[F_GRADH][i]) : TYPE == 1 ? (T)st.f[F_GRADH][i] : T(0);
        c.w = TYPE == 1 ? (T)(st.f[F_ENE][i] / p) : T(0);
    }
    rec0[i] = v;
    rec1[i] = b;
    rec2[i] = c;
    if (TYPE == 2 && gsph_2nd) {
        T* g = grad + (size_t)i * GradLayout<D>::stride;
        T v[GradLayout<D>::stride];
#pragma unroll
        for (int q = 0; q < GradLayout<D>::stride; ++q) v[q] = T(0);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            v[GradLayout<D>::d(k)] = (T)st.f[F_GRADD + k][i];
            v[GradLayout<D>::p(k)] = (T)st.f[F_GRADP + k][i];
#pragma unroll
            for (int d = 0; d < D; ++d) v[GradLayout<D>::v(k, d)] = (T)st.f[F_GRADV + 3 * k + d][i];
        }
#pragma unroll
        for (int q = 0; q < GradLayout<D>::stride; ++q) g[q] = v[q];
    }
}

}  // namespace sphgpu

// ---------------------------------------------------------------------------------------------
// Launcher (host).
namespace sphgpu {

template <int D>
constexpr int fluid_default_tile_cap() { return D == 1 ? 128 : D == 2 ? 384 : 1024; }

template <int D, typename T, int TYPE, int K>
void run_fluid(Ctx& c)
{
    using V4 = typename Vec4<T>::type;
    auto kern = fluid_kernel<D, T, TYPE, K>;
    cudaStream_t s = c.stream;
    V4* rec0 = (V4*)c.mir[2];
    V4* rec1 = (V4*)c.mir[3];
    V4* rec2 = (V4*)c.mir[4];
    T* grad = (T*)c.mir[5];
    // the records of a whole step's PreInteraction are current (it wrote them per target)
    if (!c.fluid_records_fresh)
        fluid_mirror_kernel<D, T, TYPE><<<ceil_div(c.n, 256), 256, 0, s>>>(
            c.st, c.n, rec0, rec1, rec2, grad, c.p.gsph_2nd_order, c.sound_from_ene ? c.p.gamma * (c.p.gamma - 1.0) : 0.0);
    c.fluid_records_fresh = false;
    reset_work_counters(c);
    FluidArgs<T> a{};
    a.st = c.st;
    a.tv = tree_view(c);
    a.pb = c.pb;
    a.xrel = (const V4*)c.mir[6];
    a.hmir = (const T*)c.mir[7];
    a.rec0 = rec0;
    a.rec1 = rec1;
    a.rec2 = rec2;
    a.grad = grad;
    a.gamma = c.p.gamma;
    a.gamma_t = (T)c.p.gamma;
    a.gm1_t = (T)(c.p.gamma - 1.0);
    a.alpha_ac_t = (T)c.p.alpha_ac;
    a.use_ac = c.p.use_ac;
    a.ac_gravity = c.p.use_gravity;
    a.alpha_ac = c.p.alpha_ac;
    a.gsph_2nd = c.p.gsph_2nd_order;
    a.dt_run = c.d_dt;
    a.counters = c.count_work ? c.d_counters : nullptr;
    a.bulk_stage = c.bulk_stage;
    const int tcap = c.tile_cap ? c.tile_cap : fluid_default_tile_cap<D>();
    a.pv = PlanView<T>{};
    if ((c.prewalk & 1) && c.pair_sched != 3) {
        a.pv = plan_view<T>(c);
        const int cap = first_pass_leaf_cap(c), scap = std::max(128, cap);
        a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + PLAN_WORK_SLOT, nullptr, nullptr, 0,
                           nullptr, nullptr, 0, 0, c.d_err, nullptr};
        launch_plans((const void*)fluid_walk_kernel<D, T>, c, plan_warp_bytes<T>(scap, cap),
                     [&](int grid, size_t smem) { fluid_walk_kernel<D, T><<<grid, 128, smem, c.stream>>>(a, scap, cap); });
    }
    launch_pair_passes<FluidArgs<T>>(c, (const void*)kern, a, tcap, sizeof(V4), sizeof(T),
        [](const void* k, int grid, int block, size_t smem, cudaStream_t st, FluidArgs<T>& args) {
            reinterpret_cast<void (*)(FluidArgs<T>)>(const_cast<void*>(k))<<<grid, block, smem, st>>>(args);
        },
        (const void*)fluid_tpp_kernel<D, T, TYPE, K>,
        [](const void* k, int grid, int block, cudaStream_t st, FluidArgs<T>& args) {
            reinterpret_cast<void (*)(FluidArgs<T>)>(const_cast<void*>(k))<<<grid, block, 0, st>>>(args);
        });
}

}  // namespace sphgpu
