// Group machinery shared by the pair kernels (PreInteraction, FluidForce, neighbour export).
//
// A CTA owns one target group at a time: up to blockDim.x consecutive key-ordered particles
// that the tree keeps spatially compact.  For each group the CTA
//   1. reduces the group's bounding box in FP64 (centre gc, half extent he),
//   2. walks the octree once with one warp, keeping every leaf whose box intersects the box
//      grown by the search radius (a superset of the reference's per-particle walks,
//      src/bhtree.cpp:234-270),
//   3. stages the particles of those leaves that can be in reach into a shared-memory source
//      tile: position offsets from gc computed in FP64 and stored in the pair type T, with the
//      mass in the fourth lane, plus the source's slot index, in a deterministic order,
//   4. marks per target a bitmask over the tile with the candidate predicate.
// Other per-source fields are read from key-ordered T mirror records by slot index.
// Membership predicates that decide integer results (who is a neighbour) are exact: the
// T-precision distance decides outside a guard band, and pairs inside the band are re-decided
// with the reference's own FP64 arithmetic (common.cuh: ref_r2).
//
// CTAs are persistent: each takes the next group from a device work counter until none are
// left.  A group whose walk or tile does not fit the launch's capacities is appended to an
// overflow list, which a second launch with larger capacities processes.
#pragma once

#include "common.cuh"

namespace sphgpu {

template <typename T>
struct Vec4;
template <>
struct Vec4<float> { using type = float4; };
template <>
struct Vec4<double> { using type = double4_32a; };

template <typename T>
struct Unit;
template <>
struct Unit<float> { static constexpr double u = 5.9604644775390625e-08; };   // 2^-24
template <>
struct Unit<double> { static constexpr double u = 1.1102230246251565e-16; };  // 2^-53

// Round a double to T downwards / upwards (for conservative T-precision thresholds).
template <typename T>
__device__ __forceinline__ T to_T_down(double x);
template <typename T>
__device__ __forceinline__ T to_T_up(double x);
template <>
__device__ __forceinline__ float to_T_down<float>(double x) { return __double2float_rd(x); }
template <>
__device__ __forceinline__ float to_T_up<float>(double x) { return __double2float_ru(x); }
template <>
__device__ __forceinline__ double to_T_down<double>(double x) { return x; }
template <>
__device__ __forceinline__ double to_T_up<double>(double x) { return x; }

// Shared-memory layout of a pair kernel, identical on host and device.
struct SmemLayout {
    int tcap;       // source tile capacity (multiple of 32)
    int gt;         // threads of the CTA (= targets of a group)
    int stack_cap;  // walk stack entries
    int leaf_cap;   // leaf ranges
    size_t off_stack, off_leaves, off_lpre, off_misc, off_tpos, off_tidx, off_mask, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

struct GroupMisc {
    double gc[3];
    double he[3];
    double R;           // group search radius (max over targets)
    double rmin;        // min over targets of the search radius
    double span;        // max_k he_k + R : bound on |offset| of staged sources
    double scale;       // max_k |gc_k| + max periodic length (FP64 rounding scale)
    int group;          // current group index
    int nleaves;
    int ntile;
    int overflow;
    double wred[8][8];  // per-warp reduction scratch (at most 8 warps per CTA)
};

__host__ __device__ inline SmemLayout make_layout(int gt, int tcap, int elt4, int stack_cap, int leaf_cap)
{
    SmemLayout L;
    L.tcap = tcap; L.gt = gt; L.stack_cap = stack_cap; L.leaf_cap = leaf_cap;
    size_t o = 0;
    L.off_stack = o; o = align16(o + sizeof(int) * stack_cap);
    L.off_leaves = o; o = align16(o + sizeof(int2) * leaf_cap);
    L.off_lpre = o; o = align16(o + sizeof(int) * (leaf_cap + 1));
    L.off_misc = o; o = align16(o + sizeof(GroupMisc));
    L.off_tpos = o; o = align16(o + (size_t)elt4 * tcap);
    L.off_tidx = o; o = align16(o + sizeof(int) * tcap);
    L.off_mask = o; o = align16(o + sizeof(unsigned) * (size_t)(tcap / 32) * gt);
    L.total = o;
    return L;
}

template <typename T>
struct Tile {
    typename Vec4<T>::type* pm;   // offset x, y, z from gc and mass
    int* idx;                     // key-order slot of each staged source
    unsigned* mask;               // word w of target t at mask[w * gt + t]
    int gt;
};

template <typename T>
__device__ __forceinline__ Tile<T> tile_of(unsigned char* smem, const SmemLayout& L)
{
    Tile<T> v;
    v.pm = reinterpret_cast<typename Vec4<T>::type*>(smem + L.off_tpos);
    v.idx = reinterpret_cast<int*>(smem + L.off_tidx);
    v.mask = reinterpret_cast<unsigned*>(smem + L.off_mask);
    v.gt = L.gt;
    return v;
}

// Work distribution: next group for this CTA (block-uniform), or -1 when done.
struct GroupWork {
    const int* g_begin;
    const int* g_count;
    const int* n_groups;      // number of groups (device)
    int* counter;             // work counter (device, zeroed before the launch)
    const int* list;          // optional explicit group list (overflow pass)
    const int* list_count;
    int* ovf_list;            // overflow output (main pass) or nullptr
    int* ovf_count;
    unsigned* err;
};

__device__ __forceinline__ int next_group(GroupMisc* gm, const GroupWork& w)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const int k = atomicAdd(w.counter, 1);
        int g = -1;
        if (w.list) { if (k < *w.list_count) g = w.list[k]; }
        else if (k < *w.n_groups) g = k;
        gm->group = g;
    }
    __syncthreads();
    return gm->group;
}

__device__ __forceinline__ void report_overflow(const GroupWork& w, int g)
{
    if (threadIdx.x == 0) {
        if (w.ovf_list) {
            const int k = atomicAdd(w.ovf_count, 1);
            w.ovf_list[k] = g;
        } else {
            atomicOr(w.err, (unsigned)ERR_TILE);
        }
    }
}

// ---- 1. group bounding box (FP64), block-wide ------------------------------------------------
template <int D>
__device__ void group_box(GroupMisc* gm, const double* xi, bool active, double radius, const Periodic& pb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double lo[D], hi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        lo[k] = active ? xi[k] : 1.7976931348623157e308;
        hi[k] = active ? xi[k] : -1.7976931348623157e308;
    }
    double rr = active ? radius : 0.0;
    double rm = active ? radius : 1.7976931348623157e308;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            lo[k] = fmin(lo[k], __shfl_xor_sync(FULL, lo[k], o));
            hi[k] = fmax(hi[k], __shfl_xor_sync(FULL, hi[k], o));
        }
        rr = fmax(rr, __shfl_xor_sync(FULL, rr, o));
        rm = fmin(rm, __shfl_xor_sync(FULL, rm, o));
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < D; ++k) { gm->wred[w][k] = lo[k]; gm->wred[w][3 + k] = hi[k]; }
        gm->wred[w][6] = rr;
        gm->wred[w][7] = rm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double span = 0.0, R = 0.0, sc = 0.0, Rm = 1.7976931348623157e308;
        for (int ww = 0; ww < nw; ++ww) { R = fmax(R, gm->wred[ww][6]); Rm = fmin(Rm, gm->wred[ww][7]); }
        gm->rmin = Rm;
        for (int k = 0; k < D; ++k) {
            double a = gm->wred[0][k], b = gm->wred[0][3 + k];
            for (int ww = 1; ww < nw; ++ww) { a = fmin(a, gm->wred[ww][k]); b = fmax(b, gm->wred[ww][3 + k]); }
            gm->gc[k] = 0.5 * (a + b);
            gm->he[k] = 0.5 * (b - a);
            span = fmax(span, gm->he[k]);
            sc = fmax(sc, fabs(gm->gc[k]) + (pb.on ? pb.len[k] : 0.0));
        }
        gm->R = R;
        gm->span = span + R;
        gm->scale = sc;
        gm->ntile = 0;
        gm->overflow = 0;
    }
    __syncthreads();
}

// ---- 2. tree walk by one warp -----------------------------------------------------------------
// Leaves whose box intersects [gc - he - r, gc + he + r] per axis, r = R or max(R, node kernel
// size).  Returns the number of leaves, or -1 on overflow of the stack or the leaf list.
template <int D>
__device__ int walk_group(const TreeView& tv, int root, const GroupMisc* gm, bool use_ksize,
                          const Periodic& pb, int* stack, int stack_cap, int2* leaves, int leaf_cap)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    double gc[D], he[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { gc[k] = gm->gc[k]; he[k] = gm->he[k]; }
    const double R = gm->R;
    if (lane == 0) stack[0] = root;
    int sp = 1, nl = 0;
    bool overflow = false;
    __syncwarp();
    while (sp > 0) {
        const int take = sp < 32 ? sp : 32;
        const int node = lane < take ? stack[sp - take + lane] : -1;
        __syncwarp();
        sp -= take;
        bool hit = false, leaf = false;
        int nc = 0, fc = -1;
        if (node >= 0) {
            const double e2 = 0.5 * tv.edge[node];
            const double r = use_ksize ? fmax(R, tv.ksize[node]) : R;
            hit = tv.count[node] > 0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const double d = fabs(min_image(tv.center[k][node] - gc[k], pb, k));
                const double lim = e2 + he[k] + r;
                if (d > lim * (1.0 + 1e-12)) hit = false;
            }
            fc = tv.first_child[node];
            leaf = fc < 0;
            if (hit && !leaf) nc = tv.nchild[node];
        }
        const unsigned lm = __ballot_sync(FULL, hit && leaf);
        if (hit && leaf) {
            const int pos = nl + __popc(lm & lt);
            if (pos < leaf_cap) leaves[pos] = make_int2(tv.begin[node], tv.count[node]);
        }
        nl += __popc(lm);
        int incl = nc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += t;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        if (sp + total > stack_cap) { overflow = true; break; }
        if (nc > 0) {
            const int base = sp + incl - nc;
            for (int c = 0; c < nc; ++c) stack[base + c] = fc + c;
        }
        sp += total;
        __syncwarp();
    }
    if (nl > leaf_cap) overflow = true;
    return overflow ? -1 : nl;
}

// Walk + publish the leaf count; returns false (block-uniform) on overflow.
template <int D>
__device__ bool group_walk(unsigned char* smem, const SmemLayout& L, GroupMisc* gm,
                           const TreeView& tv, int root, bool use_ksize, const Periodic& pb)
{
    if (threadIdx.x < 32) {
        int* stack = reinterpret_cast<int*>(smem + L.off_stack);
        int2* leaves = reinterpret_cast<int2*>(smem + L.off_leaves);
        const int nl = walk_group<D>(tv, root, gm, use_ksize, pb, stack, L.stack_cap, leaves, L.leaf_cap);
        if (threadIdx.x == 0) {
            gm->nleaves = nl < 0 ? 0 : nl;
            if (nl < 0) gm->overflow = 1;
        }
    }
    __syncthreads();
    return gm->overflow == 0;
}

// ---- 3. staging -------------------------------------------------------------------------------
// Flattens the leaf ranges and calls, for each particle j (key slot) in deterministic order,
// accept(j, off) where off[k] = min-image (x_j - gc) in FP64; accepted sources get consecutive
// tile slots (offsets and wval(j) stored in T).  Returns the tile count, or -1 on overflow.
template <int D, typename T, class Accept, class WVal>
__device__ int stage_sources(unsigned char* smem, const SmemLayout& L, GroupMisc* gm,
                             const State& st, const Periodic& pb, const Tile<T>& tile, Accept accept,
                             WVal wval)
{
    int2* leaves = reinterpret_cast<int2*>(smem + L.off_leaves);
    int* lpre = reinterpret_cast<int*>(smem + L.off_lpre);
    const int nl = gm->nleaves;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (w == 0) {
        int run = 0;
        for (int b = 0; b < nl; b += 32) {
            const int c = (b + lane < nl) ? leaves[b + lane].y : 0;
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            if (b + lane < nl) lpre[b + lane] = run + incl - c;
            run += __shfl_sync(FULL, incl, 31);
        }
        if (lane == 0) lpre[nl] = run;
    }
    __syncthreads();
    const int total = lpre[nl];
    int* wcnt = reinterpret_cast<int*>(&gm->wred[0][0]);
    double gc[D];
#pragma unroll
    for (int k = 0; k < D; ++k) gc[k] = gm->gc[k];
    int base = 0;
    for (int f0 = 0; f0 < total; f0 += blockDim.x) {
        const int f = f0 + threadIdx.x;
        bool ok = false;
        int j = -1;
        double off[D];
        if (f < total) {
            int lo = 0, hi = nl;   // last r with lpre[r] <= f
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (lpre[mid] <= f) lo = mid; else hi = mid;
            }
            j = leaves[lo].x + (f - lpre[lo]);
#pragma unroll
            for (int k = 0; k < D; ++k) off[k] = min_image(st.f[F_POS + k][j] - gc[k], pb, k);
            ok = accept(j, off);
        }
        const unsigned bal = __ballot_sync(FULL, ok);
        __syncthreads();   // previous iteration's readers of wcnt are done
        if (lane == 0) wcnt[w] = __popc(bal);
        __syncthreads();
        int woff = 0, tot = 0;
        for (int ww = 0; ww < nw; ++ww) {
            const int c = wcnt[ww];
            if (ww < w) woff += c;
            tot += c;
        }
        if (ok) {
            const int slot = base + woff + __popc(bal & lanemask_lt());
            if (slot < L.tcap) {
                typename Vec4<T>::type v;
                v.x = (T)off[0];
                v.y = D > 1 ? (T)off[D > 1 ? 1 : 0] : T(0);
                v.z = D > 2 ? (T)off[D > 2 ? 2 : 0] : T(0);
                v.w = wval(j);
                tile.pm[slot] = v;
                tile.idx[slot] = j;
            }
        }
        base += tot;
    }
    __syncthreads();
    return base > L.tcap ? -1 : base;
}

// ---- exact FP64 decisions for the guard band ---------------------------------------------------
template <int D>
__device__ __forceinline__ double exact_r2(const State& st, const double* xi, int j, const Periodic& pb)
{
    double xj[D];
#pragma unroll
    for (int k = 0; k < D; ++k) xj[k] = st.f[F_POS + k][j];
    return ref_r2<D>(xi, xj, pb);
}

// Guard band of |r2_T - r2_exact| for pairs with |offsets| <= span and r <= h.
template <typename T, int D>
__device__ __forceinline__ double r2_band(const GroupMisc* gm, double h)
{
    const double u = Unit<T>::u;
    const double E = u * (2.0 * gm->span + h) * 1.5 + 8.0 * Unit<double>::u * (gm->span + h + gm->scale);
    return 2.0 * 1.7320508075688772 * E * h + D * E * E + 4.0 * u * h * h;
}

// Squared distance in T between a target offset and tile source s; also returns the vector.
template <int D, typename T>
__device__ __forceinline__ T tile_r2(const T* xo, const typename Vec4<T>::type& p, T* r)
{
    r[0] = xo[0] - p.x;
    T r2 = r[0] * r[0];
    if (D > 1) { r[D > 1 ? 1 : 0] = xo[D > 1 ? 1 : 0] - p.y; r2 = fma(r[D > 1 ? 1 : 0], r[D > 1 ? 1 : 0], r2); }
    if (D > 2) { r[D > 2 ? 2 : 0] = xo[D > 2 ? 2 : 0] - p.z; r2 = fma(r[D > 2 ? 2 : 0], r[D > 2 ? 2 : 0], r2); }
    return r2;
}

}  // namespace sphgpu
