// GravityForce on the device: Barnes-Hut walk with kernel-softened particle pairs
// (GravityForce::calculation, src/gravity_force.cpp:52-89; BHTree::tree_force and
// BHNode::calc_force, src/bhtree.cpp:128-132,301-331; Hernquist & Katz (1989) softening f, g,
// src/bhtree.cpp:273-299).
//
// A warp walks the octree for 32 key-consecutive targets at once.  Each stack entry carries the
// lanes for which the node is still to be visited; every lane makes the reference's own opening
// decision for its particle (edge^2 > theta^2 |x_i - com|^2, in FP64 with the reference's
// rounding), so each particle interacts with exactly the node set of the reference's recursive
// walk: lanes that do not open a node take its monopole, lanes that open a leaf take its
// particles one by one (self term included in the potential, like the reference), lanes that
// open an inner node continue with its children.  The roots carry zero mass, as in the
// reference, whose root never receives its mass and centre (src/bhtree.cpp:57,152).
//
// FP32 pair form: leaf particles are stored as offsets from their leaf's centre in T; a lane
// forms x_i - centre once per leaf as its (two-float) x_i - com minus the record's centre - com,
// so pair separations are T differences of small numbers, and sums a leaf's terms before adding
// them to its compensated totals.  FP64 form: separations use the reference's periodic FP64
// arithmetic.  Each node is one 64-byte record (GravNode), read with four 16-byte loads.
#include "context.cuh"

namespace sphgpu {

namespace {

template <typename T>
struct GravArgs {
    using V4 = typename Vec4<T>::type;
    State st;
    TreeView tv;
    Periodic pb;
    GroupWork work;
    const V4* grel;   // {x_j - centre of j's leaf (T), m_j}: built with the tree
    const T* gh;      // h_j in T: built at the end of PreInteraction
    double G;
    double theta2;
    int stack_cap;
    unsigned long long* counters;   // PairCounter slots, or nullptr (not counted)
};

// Softened potential and force kernels (src/bhtree.cpp:273-299).
template <typename T>
__device__ __forceinline__ T hk_f(T r, T h)
{
    const T e = h * T(0.5);
    const T u = r / e;
    if (u < T(1)) {
        return (T(-0.5) * u * u * (T(1.0 / 3.0) - T(3.0 / 20) * u * u + u * u * u / T(20)) + T(1.4)) / e;
    } else if (u < T(2)) {
        return T(-1) / (T(15) * r) + (-u * u * (T(4.0 / 3.0) - u + T(0.3) * u * u - u * u * u / T(30)) + T(1.6)) / e;
    }
    return T(1) / r;
}

template <typename T>
__device__ __forceinline__ T hk_g(T r, T h)
{
    const T e = h * T(0.5);
    const T u = r / e;
    if (u < T(1)) {
        return (T(4.0 / 3.0) - T(1.2) * u * u + T(0.5) * u * u * u) / (e * e * e);
    } else if (u < T(2)) {
        const T u3 = u * u * u;
        return (T(-1.0 / 15) + T(8.0 / 3) * u3 - T(3) * u3 * u + T(1.2) * u3 * u * u - u3 * u3 / T(6.0)) / (r * r * r);
    }
    return T(1) / (r * r * r);
}

// COUNT: a separate instantiation counts the monopole terms and leaf pairs (knob 25), so that the
// timed kernel carries no counter registers.
template <int D, typename T, bool COUNT>
__global__ void __launch_bounds__(256) gravity_kernel(GravArgs<T> a)
{
    using V4 = typename Vec4<T>::type;
    extern __shared__ __align__(16) int2 gstack[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int2* stack = gstack + (size_t)w * a.stack_cap;
    const State& st = a.st;
    const TreeView& tv = a.tv;
    const T G = (T)a.G;
    constexpr bool exact_pairs = sizeof(T) == 8;

    // each warp takes its own work items (32 targets of a group) from the counter: warps share no
    // data, so none waits at a barrier for the slowest walk of its block
    for (;;) {
        int k = 0;
        // no more work once the octree of this step is known to be incomplete (checked per work
        // item: a check at kernel entry kept four more registers live, one block fewer per SM)
        if (lane == 0) k = tree_failed(a.work.err) ? 0x7fffffff : atomicAdd(a.work.counter, 1);
        k = __shfl_sync(FULL, k, 0);
        const int g = k / a.work.pieces, o = 32 * (k % a.work.pieces);
        if (g >= *a.work.n_groups) break;
        const int gb = a.work.g_begin[g], gn = a.work.g_count[g];
        if (o >= gn) continue;
        const int t = o + lane;
        const bool active = t < gn;
        const int i = gb + (active ? t : 0);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = st.f[F_POS + k][i];
        const double hi = st.f[F_SML][i];
        const T hiT = (T)hi;
        // FP32 opening test (FP32 pair form): x_i and the centres of mass in FP32 differ from the
        // exact values by at most u (|x| + |com| + |d|) per component; xmag bounds |x| (plus a
        // periodic length), which the test's margin scales with.
        // x_i as a two-float pair: for nearby points hi_i - hi_c is exact in FP32 (Sterbenz), so
        // (hi_i - hi_c) + (lo_i - lo_c) reproduces x_i - c to FP32 rounding of the difference.
        float xf[D], xlo[D];
        float xmag = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            xf[k] = (float)xi[k];
            xlo[k] = (float)(xi[k] - (double)xf[k]);
            xmag = fmaxf(xmag, fabsf(xf[k]) + (a.pb.on ? a.pb.lenf[k] : 0.f));
        }
        const float theta2f = (float)a.theta2;
        Sum<T> phi, acc[D];
        phi.zero();
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k].zero();

        unsigned n_mono = 0, n_pair = 0;   // work counts of this lane (knob 25)
        const unsigned amask = __ballot_sync(FULL, active);
        if (lane == 0) stack[0] = make_int2(st.run[gb], (int)amask);
        int sp = 1;
        bool overflow = false;
        __syncwarp();
        while (sp > 0) {
            const int2 e = stack[sp - 1];
            --sp;
            __syncwarp();
            const int node = e.x;
            const unsigned m = (unsigned)e.y;
            const bool in = (m >> lane) & 1u;
            // the whole record at once (one latency for the node instead of one per field)
            const GravNode* gp = tv.gn + node;
            const int4 link = gp->link;
            float4 gcom, gcomlo, gcc;
            if (!exact_pairs) {
                gcom = gp->com;
                gcomlo = gp->comlo;
                gcc = gp->cc;
            }
            bool open = false;
            float df[D] = {};
            if (in) {
                T dT[D];
                bool decided = false;
                if (!exact_pairs) {
                    // edge^2 > theta^2 |d|^2 in FP32, certain outside the margin
                    const float cx[3] = {gcom.x, gcom.y, gcom.z}, cl[3] = {gcomlo.x, gcomlo.y, gcomlo.z};
                    float d2f = 0.f;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        df[k] = min_image_f((xf[k] - cx[k]) + (xlo[k] - cl[k]), a.pb, k);
                        d2f = fmaf(df[k], df[k], d2f);
                    }
                    const float l2 = gcom.w;
                    const float dabs = sqrtf(d2f);
                    const float u = 5.9604645e-08f;
                    const float margin = theta2f * (8.f * u * dabs * (xmag + dabs) + 8.f * u * d2f) + 8.f * u * l2;
                    const float t2d2 = theta2f * d2f;
                    if (l2 > t2d2 + margin) { open = true; decided = true; }
                    else if (l2 < t2d2 - margin) { open = false; decided = true; }
#pragma unroll
                    for (int k = 0; k < D; ++k) dT[k] = (T)df[k];
                }
                if (!decided) {
                    // the reference's FP64 test (src/bhtree.cpp:304-308)
                    double d[D];
#pragma unroll
                    for (int k = 0; k < D; ++k) d[k] = ref_axis(xi[k], tv.com[k][node], a.pb, k);
                    double d2 = __dmul_rn(d[0], d[0]);
#pragma unroll
                    for (int k = 1; k < D; ++k) d2 = __dadd_rn(d2, __dmul_rn(d[k], d[k]));
                    const double edge = tv.edge[node];
                    open = __dmul_rn(edge, edge) > __dmul_rn(a.theta2, d2);
#pragma unroll
                    for (int k = 0; k < D; ++k) dT[k] = (T)d[k];
                }
                if (!open) {
                    const T M = exact_pairs ? (T)tv.mass[node] : (T)gcomlo.w;
                    if (M != T(0)) {
                        if (COUNT) ++n_mono;
                        // monopole: phi -= G M / r, acc -= d G M / r^3 (src/bhtree.cpp:327-329)
                        T r2 = T(0);
#pragma unroll
                        for (int k = 0; k < D; ++k) r2 += dT[k] * dT[k];
                        const T r_inv = rsqrt_t(r2);
                        const T gmr = G * (T)M * r_inv;
                        phi.add(-gmr);
                        const T c = gmr * r_inv * r_inv;
#pragma unroll
                        for (int k = 0; k < D; ++k) acc[k].add(-dT[k] * c);
                    }
                }
            }
            const unsigned om = __ballot_sync(FULL, open);
            if (!om) continue;
            const int fc = link.x;
            if (fc < 0 && !exact_pairs && __popc(om) * link.w <= 32) {
                // a leaf that few lanes open, transposed: lane q evaluates pair (t, j) = (q / cnt,
                // b + q % cnt) for the t-th opening lane, the pairs of one target are summed by a
                // segmented shuffle reduction, and each opening lane adds its leaf sum to its
                // compensated totals (cnt iterations with a few active lanes become one with all)
                const int b = link.z, cnt = link.w;
                const int kopen = __popc(om);
                if (COUNT && open) n_pair += (unsigned)cnt;
                T base[D];
                {
                    const float cc[3] = {gcc.x, gcc.y, gcc.z};
#pragma unroll
                    for (int k = 0; k < D; ++k) base[k] = (T)min_image_f(df[k] - cc[k], a.pb, k);
                }
                const bool pv = lane < kopen * cnt;
                const int t = pv ? lane / cnt : 0;
                unsigned mm = om;
                for (int z = 0; z < t; ++z) mm &= mm - 1;
                const int src = pv ? __ffs(mm) - 1 : 0;
                T bt[D];
#pragma unroll
                for (int k = 0; k < D; ++k) bt[k] = __shfl_sync(FULL, base[k], src);
                const T hit = __shfl_sync(FULL, hiT, src);
                T pphi = T(0), pacc[D];
#pragma unroll
                for (int k = 0; k < D; ++k) pacc[k] = T(0);
                if (pv) {
                    const int j = b + (lane - t * cnt);
                    const V4 q = a.grel[j];
                    const T hj = a.gh[j];
                    T rv[D];
                    rv[0] = bt[0] - q.x;
                    if (D > 1) rv[D > 1 ? 1 : 0] = bt[D > 1 ? 1 : 0] - q.y;
                    if (D > 2) rv[D > 2 ? 2 : 0] = bt[D > 2 ? 2 : 0] - q.z;
                    T r2 = rv[0] * rv[0];
#pragma unroll
                    for (int k = 1; k < D; ++k) r2 += rv[k] * rv[k];
                    T fsum, gsum;
                    const T hmax = hit > hj ? hit : hj;
                    if (r2 >= hmax * hmax && r2 > T(0)) {
                        const T rinv = rsqrt_t(r2);
                        fsum = T(2) * rinv;
                        gsum = fsum * rinv * rinv;
                    } else {
                        const T r = sqrt(r2);
                        fsum = hk_f(r, hit) + hk_f(r, hj);
                        gsum = hk_g(r, hit) + hk_g(r, hj);
                    }
                    const T gm = G * q.w * T(0.5);
                    pphi = -gm * fsum;
                    const T c = gm * gsum;
#pragma unroll
                    for (int k = 0; k < D; ++k) pacc[k] = -rv[k] * c;
                }
                // segmented sums over [t cnt, (t + 1) cnt): the segment's first lane ends with them
                const int seg_end = pv ? (t + 1) * cnt : lane + 1;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const bool in_seg = lane + o < seg_end;
                    const T vphi = __shfl_down_sync(FULL, pphi, o);
                    if (in_seg) pphi += vphi;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const T v = __shfl_down_sync(FULL, pacc[k], o);
                        if (in_seg) pacc[k] += v;
                    }
                }
                const int from = open ? __popc(om & lanemask_lt()) * cnt : 0;
                const T sphi = __shfl_sync(FULL, pphi, from);
                T sacc[D];
#pragma unroll
                for (int k = 0; k < D; ++k) sacc[k] = __shfl_sync(FULL, pacc[k], from);
                if (open) {
                    phi.add(sphi);
#pragma unroll
                    for (int k = 0; k < D; ++k) acc[k].add(sacc[k]);
                }
            } else if (fc < 0) {
                if (open) {
                    const int b = link.z, cnt = link.w;
                    if (COUNT) n_pair += (unsigned)cnt;
                    T base[D];
                    if (!exact_pairs) {
                        // x_i - centre = (x_i - com) - (centre - com)
                        const float cc[3] = {gcc.x, gcc.y, gcc.z};
#pragma unroll
                        for (int k = 0; k < D; ++k) base[k] = (T)min_image_f(df[k] - cc[k], a.pb, k);
                    }
                    // the leaf's terms summed plainly, then added to the compensated totals once
                    T lphi = T(0), lacc[D];
#pragma unroll
                    for (int k = 0; k < D; ++k) lacc[k] = T(0);
                    V4 qn{};
                    T hn = T(0);
                    if (!exact_pairs) { qn = a.grel[b]; hn = a.gh[b]; }
                    for (int j = b; j < b + cnt; ++j) {
                        T rv[D], mj, hj;
                        if (exact_pairs) {
#pragma unroll
                            for (int k = 0; k < D; ++k) rv[k] = (T)ref_axis(xi[k], st.f[F_POS + k][j], a.pb, k);
                            mj = (T)st.f[F_MASS][j];
                            hj = (T)st.f[F_SML][j];
                        } else {
                            // the next particle's record is loaded before this one is evaluated
                            const V4 q = qn;
                            hj = hn;
                            if (j + 1 < b + cnt) { qn = a.grel[j + 1]; hn = a.gh[j + 1]; }
                            rv[0] = base[0] - q.x;
                            if (D > 1) rv[D > 1 ? 1 : 0] = base[D > 1 ? 1 : 0] - q.y;
                            if (D > 2) rv[D > 2 ? 2 : 0] = base[D > 2 ? 2 : 0] - q.z;
                            mj = q.w;
                        }
                        T r2 = rv[0] * rv[0];
#pragma unroll
                        for (int k = 1; k < D; ++k) r2 += rv[k] * rv[k];
                        T fsum, gsum;
                        const T hmax = hiT > hj ? hiT : hj;
                        if (r2 >= hmax * hmax && r2 > T(0)) {
                            // beyond both softening lengths (u = 2 r / h >= 2 for h_i and h_j):
                            // f = 1/r and g = 1/r^3 for both (src/bhtree.cpp:282-283,296-297)
                            const T rinv = rsqrt_t(r2);
                            fsum = T(2) * rinv;
                            gsum = fsum * rinv * rinv;
                        } else {
                            const T r = sqrt(r2);
                            fsum = hk_f(r, hiT) + hk_f(r, hj);
                            gsum = hk_g(r, hiT) + hk_g(r, hj);
                        }
                        const T gm = G * mj * T(0.5);
                        if (exact_pairs) {
                            phi.add(-gm * fsum);
                        } else {
                            lphi -= gm * fsum;
                        }
                        const T c = gm * gsum;
#pragma unroll
                        for (int k = 0; k < D; ++k) {
                            if (exact_pairs) acc[k].add(-rv[k] * c);
                            else lacc[k] -= rv[k] * c;
                        }
                    }
                    if (!exact_pairs) {
                        phi.add(lphi);
#pragma unroll
                        for (int k = 0; k < D; ++k) acc[k].add(lacc[k]);
                    }
                }
            } else {
                const int nc = link.y;
                if (sp + nc > a.stack_cap) { overflow = true; break; }
                if (lane < nc) {
                    stack[sp + nc - 1 - lane] = make_int2(fc + lane, (int)om);
                    // the children's records come in while the first child's subtree is walked
                    prefetch_l1(tv.gn + fc + lane);
                }
                sp += nc;
                __syncwarp();
            }
        }
        if (overflow) {
            if (lane == 0) atomicOr(a.work.err, (unsigned)ERR_GSTACK);
            continue;
        }
        if (COUNT) {
            warp_count(a.counters + PC_GRAV_NODES, active ? n_mono : 0u);
            warp_count(a.counters + PC_GRAV_PAIRS, active ? n_pair : 0u);
        }
        if (active) {
#pragma unroll
            for (int k = 0; k < D; ++k) st.f[F_ACC + k][i] += (double)acc[k].get();
            st.f[F_PHI][i] = (double)phi.get();
        }
    }
}

template <int D, typename T>
void run_gravity(Ctx& c)
{
    using V4 = typename Vec4<T>::type;
    cudaStream_t s = c.stream;
    V4* grel = (V4*)c.mir[6];
    T* gh = (T*)c.mir[7];
    TreeView tv = tree_view(c);
    reset_work_counters(c);
    GravArgs<T> a{};
    a.st = c.st;
    a.tv = tv;
    a.pb = c.pb;
    a.grel = grel;
    a.gh = gh;
    a.G = c.p.g_constant;
    a.theta2 = c.p.theta * c.p.theta;
    // deepest stack: 2^D - 1 siblings waiting per level below the root, plus one node's children
    a.stack_cap = 256;
    a.counters = c.count_work ? c.d_counters : nullptr;
    if (c.gravity_items == 1 && c.d_gchunk_begin) {
        a.work = GroupWork{c.d_gchunk_begin, c.d_gchunk_count, c.d_gchunk_n, c.d_work + 0, nullptr, nullptr, 0,
                           nullptr, nullptr, 0, 0, c.d_err, nullptr};
        a.work.pieces = 1;
    } else {
        a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + 0, nullptr, nullptr, 0, nullptr,
                           nullptr, 0, 0, c.d_err, nullptr};
        a.work.pieces = c.group_threads / 32;
    }
    const int gt = 128;   // four independent warps per block
    const size_t smem = sizeof(int2) * (size_t)a.stack_cap * (gt / 32);
    auto kern = a.counters ? gravity_kernel<D, T, true> : gravity_kernel<D, T, false>;
    cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int nb = std::max(1, kernel_occupancy((const void*)kern, gt, smem));
    kern<<<nb * c.num_sms, gt, smem, s>>>(a);
}

}  // namespace

void launch_gravity(Ctx& c)
{
    const bool f32 = c.precision == SPHGPU_FP32_PAIR;
    if (c.dim == 1) { if (f32) run_gravity<1, float>(c); else run_gravity<1, double>(c); }
    else if (c.dim == 2) { if (f32) run_gravity<2, float>(c); else run_gravity<2, double>(c); }
    else { if (f32) run_gravity<3, float>(c); else run_gravity<3, double>(c); }
}

}  // namespace sphgpu
