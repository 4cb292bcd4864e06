// Group machinery shared by the pair kernels (PreInteraction, FluidForce, neighbour export).
//
// A CTA owns one target group at a time: G key-consecutive particles of one run (a fixed chunk
// of the key order, which the octree keeps spatially compact).  For each group the CTA
//   1. reduces the group's bounding box in FP64 (centre gc, half extent he) and the search
//      radius R = max over targets,
//   2. walks the octree once with one warp in FP32 with conservative margins, keeping every
//      leaf whose box can intersect the box grown by the search radius (a superset of the
//      reference's per-particle walks, src/bhtree.cpp:234-270); for each kept leaf it forms the
//      offset of the leaf centre from gc once in FP64,
//   3. stages the particles of those leaves that can be in reach into a shared-memory source
//      tile: offset from gc = (leaf centre - gc) + (x_j - leaf centre), the second term read from
//      a per-particle mirror in T, so no FP64 arithmetic is done per source; mass and one
//      auxiliary value per source go along, plus the source's key-order slot,
//   4. marks per target a bitmask over the tile with a candidate predicate.
// Other per-source fields are read from key-ordered T mirror records by slot index.
// Membership predicates that decide integer results (who is a neighbour) are exact: the
// T-precision distance decides outside a guard band that bounds its rounding error, and pairs
// inside the band are re-decided with the reference's own FP64 arithmetic (common.cuh: ref_r2).
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
    size_t off_stack, off_leaves, off_loff, off_lpre, off_misc, off_tpos, off_taux, off_tidx,
        off_mask, off_wbox, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

struct GroupMisc {
    unsigned long long mbar;   // mbarrier of the bulk-copy staging (initialised by bulk_stage_init)
    unsigned mbar_phase;       // parity of its current phase
    double gc[3];
    double he[3];
    double R;           // group search radius (max over targets)
    double rmin;        // min over targets of the search radius
    double span;        // max_k he_k + R : bound on |offset| of staged sources
    double scale;       // max_k |gc_k| + max periodic length (FP64 rounding scale)
    double bmax;        // max half-diagonal of the walked leaves (bound on |x_j - leaf centre|)
    float gcf[3];       // gc in FP32
    float hef[3];       // he rounded up
    float Rf;           // R rounded up
    int group;          // current group index
    int nleaves;
    int ntile;
    int overflow;
    int gidx;           // index of the current work item in the group list (-1: a range of a later pass)
    float bandf;        // a pair kernel's relative guard band of the group, formed once (FP32 / FP64 form)
    double bandd;
    double wred[8][8];  // per-warp reduction scratch (at most 8 warps per CTA)
};

// A group's box and walked leaves, formed for a pair kernel's first pass by walk_groups_kernel:
// the GroupMisc fields that group_box and walk_group set, and where its leaves lie in the pool.
struct GroupPlan {
    double gc[3], he[3];
    double R, rmin, span, scale, bmax;
    float gcf[3], hef[3];
    float Rf;
    int nleaves;        // -1: the walk overflowed its capacities; -2: no room in the pool (walk in the pair kernel)
    int leaf_off;       // first entry of the group's leaves in the pool
};

// Where walk_groups_kernel leaves its plans (plans for the first plan_cap groups of the list; the
// leaves of all of them in one pool, taken by an atomic counter).
template <typename T>
struct PlanView {
    GroupPlan* plan;                 // nullptr: no plans (the pair kernels walk themselves)
    int plan_cap;
    int2* leaves;                    // pool: (begin, count) of each leaf
    typename Vec4<T>::type* loff;    // pool: leaf centre offsets from the group centre
    int pool_cap;
    int* pool_count;                 // device counter of the pool
};

// elt4 = sizeof(Vec4<T>), eltT = sizeof(T)
__host__ __device__ inline SmemLayout make_layout(int gt, int tcap, int elt4, int eltT, int stack_cap,
                                                  int leaf_cap)
{
    SmemLayout L;
    L.tcap = tcap; L.gt = gt; L.stack_cap = stack_cap; L.leaf_cap = leaf_cap;
    size_t o = 0;
    L.off_stack = o; o = align16(o + sizeof(int) * stack_cap);
    L.off_leaves = o; o = align16(o + sizeof(int2) * leaf_cap);
    L.off_loff = o; o = align16(o + (size_t)elt4 * leaf_cap);
    L.off_lpre = o; o = align16(o + sizeof(int) * (leaf_cap + 1));
    L.off_misc = o; o = align16(o + sizeof(GroupMisc));
    L.off_tpos = o; o = align16(o + (size_t)elt4 * tcap);
    L.off_taux = o; o = align16(o + (size_t)eltT * tcap);
    L.off_tidx = o; o = align16(o + sizeof(int) * tcap);
    L.off_mask = o; o = align16(o + sizeof(unsigned) * (size_t)(tcap / 32) * gt);
    L.off_wbox = o; o = align16(o + (size_t)elt4 * 2 * (size_t)(tcap / 32));
    L.total = o;
    return L;
}

template <typename T>
struct Tile {
    typename Vec4<T>::type* pm;   // offset x, y, z from gc and mass
    T* aux;                       // one auxiliary value per source (stage-defined)
    int* idx;                     // key-order slot of each staged source
    unsigned* mask;               // word w of target t at mask[w * gt + t]
    // bounding box of the offsets of the 32 sources of mask word w: wbox[2 w] = {min x, min y,
    // min z, min aux}, wbox[2 w + 1] = {max x, max y, max z, max aux}
    typename Vec4<T>::type* wbox;
    int gt;
};

template <typename T>
__device__ __forceinline__ Tile<T> tile_of(unsigned char* smem, const SmemLayout& L)
{
    Tile<T> v;
    v.pm = reinterpret_cast<typename Vec4<T>::type*>(smem + L.off_tpos);
    v.aux = reinterpret_cast<T*>(smem + L.off_taux);
    v.idx = reinterpret_cast<int*>(smem + L.off_tidx);
    v.mask = reinterpret_cast<unsigned*>(smem + L.off_mask);
    v.wbox = reinterpret_cast<typename Vec4<T>::type*>(smem + L.off_wbox);
    v.gt = L.gt;
    return v;
}

// Squared distance in T from a target offset to the box of mask word w (3D tiles; 0 otherwise,
// i.e. no word is skipped).  It is formed with the
// operations of tile_r2 on per-axis distances that are never larger than the word's sources'
// (rounding is monotonic), so it never exceeds tile_r2 of any source of the word: a word whose
// box distance already fails a target's test holds no source that passes it.
template <int D, typename T>
__device__ __forceinline__ T word_box_r2(const T* xo, const Tile<T>& tile, int w)
{
    if (D != 3) return T(0);
    const typename Vec4<T>::type lo = tile.wbox[2 * w], hi = tile.wbox[2 * w + 1];
    const T l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
    T d[3];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const T a = l[k] - xo[k], b = xo[k] - h[k];
        const T m = a > b ? a : b;
        d[k] = m > T(0) ? m : T(0);
    }
    T r2 = d[0] * d[0];
    if (D > 1) r2 = fma(d[D > 1 ? 1 : 0], d[D > 1 ? 1 : 0], r2);
    if (D > 2) r2 = fma(d[D > 2 ? 2 : 0], d[D > 2 ? 2 : 0], r2);
    return r2;
}

// The set bits of one target's candidate mask, visited across all words in one loop, so that a
// warp runs max-over-lanes of the candidate counts (not the sum over words of per-word maxima).
struct MaskIter {
    unsigned* mask;
    int gt, t, nw, w, b;
    unsigned bits;
    __device__ __forceinline__ MaskIter(unsigned* m, int gt_, int t_, int nw_, unsigned long long = ~0ull)
        : mask(m), gt(gt_), t(t_), nw(nw_), w(0), b(0), bits(nw_ > 0 ? m[t_] : 0u) {}
    __device__ __forceinline__ bool next(int& s)
    {
        while (bits == 0) {
            if (++w >= nw) return false;
            bits = mask[w * gt + t];
        }
        b = __ffs(bits) - 1;
        bits &= bits - 1;
        s = w * 32 + b;
        return true;
    }
    // drop the source last returned by next() from the stored mask
    __device__ __forceinline__ void clear_current() { mask[w * gt + t] &= ~(1u << b); }
    // drop source s (returned by an earlier next()) from the stored mask
    __device__ __forceinline__ void clear(int s) { mask[(s >> 5) * gt + t] &= ~(1u << (s & 31)); }
};

// MaskIter over the words that hold candidates only (bit w of `words`, recorded while the mask
// was built; tiles of at most 64 words), loading the next such word's bits while the current one
// is consumed.  Larger tiles scan every word in turn.  It costs a few registers more than MaskIter.
struct MaskWordIter {
    unsigned* mask;
    int gt, t, nw, w, b;
    unsigned bits;
    unsigned long long wm;   // words still to visit after pw
    int pw;                  // next word to visit (-1: none)
    unsigned pbits;          // its bits, loaded ahead
    __device__ __forceinline__ MaskWordIter(unsigned* m, int gt_, int t_, int nw_, unsigned long long words)
        : mask(m), gt(gt_), t(t_), nw(nw_), w(-1), b(0), bits(0u), pw(-1), pbits(0u)
    {
        wm = nw_ > 64 ? 0ull : (words & (nw_ == 64 ? ~0ull : ((1ull << nw_) - 1ull)));
        advance();
    }
    __device__ __forceinline__ void advance()
    {
        if (wm) {
            pw = __ffsll((long long)wm) - 1;
            wm &= wm - 1;
            pbits = mask[pw * gt + t];
        } else {
            pw = -1;
        }
    }
    __device__ __forceinline__ bool next(int& s)
    {
        while (bits == 0) {
            if (nw > 64) {
                if (++w >= nw) return false;
                bits = mask[w * gt + t];
                continue;
            }
            if (pw < 0) return false;
            w = pw;
            bits = pbits;
            advance();
        }
        b = __ffs(bits) - 1;
        bits &= bits - 1;
        s = w * 32 + b;
        return true;
    }
    __device__ __forceinline__ void clear(int s) { mask[(s >> 5) * gt + t] &= ~(1u << (s & 31)); }
    // the next word holding candidates and its bits (a word-level walk; do not mix with next())
    __device__ __forceinline__ bool next_word(int& wo, unsigned& bo)
    {
        if (nw > 64) {
            while (++w < nw) {
                const unsigned m = mask[w * gt + t];
                if (m) { wo = w; bo = m; return true; }
            }
            return false;
        }
        if (pw < 0) return false;
        wo = pw;
        bo = pbits;
        advance();
        return true;
    }
};

// Work distribution.  A work item is a range of key-consecutive targets (begin, count).  The
// first pass takes the group list; later passes take the ranges earlier passes could not fit.
struct GroupWork {
    const int* g_begin;
    const int* g_count;
    const int* n_groups;      // number of groups (device)
    int* counter;             // work counter (device, zeroed before the launch)
    const int2* list;         // ranges left by the previous pass (nullptr in the first pass)
    const int* list_count;
    int list_cap;             // capacity of both range lists
    int2* ovf_list;           // ranges this pass cannot fit (nullptr in the last pass)
    int* ovf_count;
    int ovf_cap;
    int halve;                // pass a failing range on as its two halves
    unsigned* err;
    int* fail_info;           // last pass: {begin, count, R in units of 1e-9, leaves, sources}
    int pieces = 1;           // thread-per-particle kernels: work items of 32 targets per range
};

// Next work item for this CTA (block-uniform); false when done.
__device__ __forceinline__ bool next_group(GroupMisc* gm, const GroupWork& w, int& gb, int& gn)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const int k = atomicAdd(w.counter, 1);
        int b = -1, n = 0;
        if (w.list) {
            if (k < min(*w.list_count, w.list_cap)) { const int2 r = w.list[k]; b = r.x; n = r.y; }
        } else if (k < *w.n_groups) {
            b = w.g_begin[k];
            n = w.g_count[k];
        }
        gm->group = b;
        gm->ntile = n;   // scratch: the range length
        gm->gidx = w.list ? -1 : k;
    }
    __syncthreads();
    gb = gm->group;
    gn = gm->ntile;
    return gb >= 0;
}

__device__ __forceinline__ void push_range(const GroupWork& w, int b, int n)
{
    const int k = atomicAdd(w.ovf_count, 1);
    if (k < w.ovf_cap) w.ovf_list[k] = make_int2(b, n);
    else atomicOr(w.err, (unsigned)ERR_TILE);
}

__device__ __forceinline__ void report_overflow(const GroupWork& w, int gb, int gn, const GroupMisc* gm = nullptr)
{
    if (threadIdx.x == 0) {
        if (!w.ovf_list) {
            atomicOr(w.err, (unsigned)ERR_TILE);
            if (w.fail_info && gm) {
                w.fail_info[0] = gb;
                w.fail_info[1] = gn;
                w.fail_info[2] = (int)fmin(gm->R * 1e9, 2e9);
                w.fail_info[3] = gm->nleaves;
                w.fail_info[4] = gm->overflow;
            }
        } else if (w.halve && gn > 1) {
            push_range(w, gb, gn / 2);
            push_range(w, gb + gn / 2, gn - gn / 2);
        } else {
            push_range(w, gb, gn);
        }
    }
}

// ---- 1. group bounding box (FP64), block-wide ------------------------------------------------
// The box fields from the targets' coordinate minima lo and maxima hi, the largest search radius R
// and the smallest Rm (one thread).
template <int D>
__device__ __forceinline__ void finish_box(GroupMisc* gm, const double* lo, const double* hi, double R, double Rm,
                                           const Periodic& pb)
{
    double span = 0.0, sc = 0.0;
    gm->rmin = Rm;
    for (int k = 0; k < D; ++k) {
        const double a = lo[k], b = hi[k];
        gm->gc[k] = 0.5 * (a + b);
        // half extent, rounded so that every target lies within gc +/- he
        gm->he[k] = fmax(b - gm->gc[k], gm->gc[k] - a);
        span = fmax(span, gm->he[k]);
        sc = fmax(sc, fabs(gm->gc[k]) + (pb.on ? pb.len[k] : 0.0));
        gm->gcf[k] = (float)gm->gc[k];
        gm->hef[k] = __double2float_ru(gm->he[k]);
    }
    gm->R = R;
    gm->Rf = __double2float_ru(R);
    gm->span = span + R;
    gm->scale = sc;
    gm->bmax = 0.0;
    gm->ntile = 0;
    gm->overflow = 0;
}

template <int D>
__device__ void group_box(GroupMisc* gm, const double* xi, bool active, double radius, const Periodic& pb)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // minima and maxima on the ordered-integer images of the doubles (exact, and off the FP64
    // pipe, which runs at 1/64 of the FP32 rate)
    const long long top = dbl_to_ord(1.7976931348623157e308), bottom = dbl_to_ord(-1.7976931348623157e308);
    long long lo[D], hi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const long long o = dbl_to_ord(xi[k]);
        lo[k] = active ? o : top;
        hi[k] = active ? o : bottom;
    }
    long long rr = active ? dbl_to_ord(radius) : 0;
    long long rm = active ? dbl_to_ord(radius) : top;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            lo[k] = min(lo[k], __shfl_xor_sync(FULL, lo[k], o));
            hi[k] = max(hi[k], __shfl_xor_sync(FULL, hi[k], o));
        }
        rr = max(rr, __shfl_xor_sync(FULL, rr, o));
        rm = min(rm, __shfl_xor_sync(FULL, rm, o));
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < D; ++k) { gm->wred[w][k] = ord_to_dbl(lo[k]); gm->wred[w][3 + k] = ord_to_dbl(hi[k]); }
        gm->wred[w][6] = ord_to_dbl(rr);
        gm->wred[w][7] = ord_to_dbl(rm);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double R = 0.0, Rm = 1.7976931348623157e308, lo_[3] = {0.0, 0.0, 0.0}, hi_[3] = {0.0, 0.0, 0.0};
        for (int ww = 0; ww < nw; ++ww) { R = fmax(R, gm->wred[ww][6]); Rm = fmin(Rm, gm->wred[ww][7]); }
        for (int k = 0; k < D; ++k) {
            double a = gm->wred[0][k], b = gm->wred[0][3 + k];
            for (int ww = 1; ww < nw; ++ww) { a = fmin(a, gm->wred[ww][k]); b = fmax(b, gm->wred[ww][3 + k]); }
            lo_[k] = a;
            hi_[k] = b;
        }
        finish_box<D>(gm, lo_, hi_, R, Rm, pb);
    }
    __syncthreads();
}

// ---- 2. tree walk by one warp, in FP32 -----------------------------------------------------------
// Leaves whose box can intersect [gc - he - r, gc + he + r] per axis, r = R or max(R, node
// kernel size).  The FP32 test keeps a node whenever the exact test might: the rounding of
// centre, gc and their difference is below 3u (|gc| + d), covered by the relative margin and the
// absolute slack.  For each kept leaf the offset of its centre from gc is formed in FP64 and
// stored in T.  Returns the number of leaves, or -1 on overflow of the stack or the leaf list.
template <int D, typename T>
__device__ int walk_group(const TreeView& tv, int root, GroupMisc* gm, bool use_ksize,
                          const Periodic& pb, int* stack, int stack_cap, int2* leaves,
                          typename Vec4<T>::type* loff, int leaf_cap)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    float gcf[D], hef[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { gcf[k] = gm->gcf[k]; hef[k] = gm->hef[k]; }
    const float Rf = gm->Rf;
    const float slack = (float)(4.0 * 5.9604644775390625e-08 * gm->scale) + 1e-30f;
    if (lane == 0) stack[0] = root;
    int sp = 1, nl = 0;
    bool overflow = false;
    float bmax = 0.f;
    __syncwarp();
    while (sp > 0) {
        const int take = sp < 32 ? sp : 32;
        const int node = lane < take ? stack[sp - take + lane] : -1;
        __syncwarp();
        sp -= take;
        bool hit = false, leaf = false;
        int nc = 0, fc = -1;
        if (node >= 0) {
            const float e2 = 0.5f * tv.ef[node];
            const float r = use_ksize ? fmaxf(Rf, tv.kf[node]) : Rf;
            hit = tv.count[node] > 0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const float d = fabsf(min_image_f(tv.cf[k][node] - gcf[k], pb, k));
                const float lim = e2 + hef[k] + r;
                if (d > lim * 1.00001f + slack) hit = false;
            }
            fc = tv.first_child[node];
            leaf = fc < 0;
            if (hit && !leaf) nc = tv.nchild[node];
        }
        const unsigned lm = __ballot_sync(FULL, hit && leaf);
        if (hit && leaf) {
            const int pos = nl + __popc(lm & lt);
            if (pos < leaf_cap) {
                leaves[pos] = make_int2(tv.begin[node], tv.count[node]);
                typename Vec4<T>::type o;
                o.x = (T)min_image(tv.center[0][node] - gm->gc[0], pb, 0);
                o.y = D > 1 ? (T)min_image(tv.center[D > 1 ? 1 : 0][node] - gm->gc[D > 1 ? 1 : 0], pb, D > 1 ? 1 : 0) : T(0);
                o.z = D > 2 ? (T)min_image(tv.center[D > 2 ? 2 : 0][node] - gm->gc[D > 2 ? 2 : 0], pb, D > 2 ? 2 : 0) : T(0);
                o.w = T(0);
                loff[pos] = o;
            }
            bmax = fmaxf(bmax, tv.ef[node]);
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
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bmax = fmaxf(bmax, __shfl_xor_sync(FULL, bmax, o));
    if (lane == 0) gm->bmax = 0.5 * (double)bmax * 1.7320508075688772 * (1.0 + 1e-6);
    if (nl > leaf_cap) overflow = true;
    return overflow ? -1 : nl;
}

// Walk + publish the leaf count; returns false (block-uniform) on overflow.
template <int D, typename T>
__device__ bool group_walk(unsigned char* smem, const SmemLayout& L, GroupMisc* gm,
                           const TreeView& tv, int root, bool use_ksize, const Periodic& pb)
{
    if (threadIdx.x < 32) {
        int* stack = reinterpret_cast<int*>(smem + L.off_stack);
        int2* leaves = reinterpret_cast<int2*>(smem + L.off_leaves);
        auto* loff = reinterpret_cast<typename Vec4<T>::type*>(smem + L.off_loff);
        const int nl = walk_group<D, T>(tv, root, gm, use_ksize, pb, stack, L.stack_cap, leaves, loff, L.leaf_cap);
        if (threadIdx.x == 0) {
            gm->nleaves = nl < 0 ? 0 : nl;
            if (nl < 0) gm->overflow = 1;
        }
    }
    __syncthreads();
    return gm->overflow == 0;
}

// Shared memory of one warp of walk_groups_kernel: its GroupMisc, walk stack, leaves and offsets.
template <typename T>
__host__ __device__ inline size_t plan_warp_bytes(int stack_cap, int cap)
{
    return align16(sizeof(GroupMisc)) + align16(sizeof(int) * (size_t)stack_cap) + align16(sizeof(int2) * (size_t)cap) +
           align16(sizeof(typename Vec4<T>::type) * (size_t)cap);
}

// One warp per group of the list, ahead of a pair kernel's first pass: the group box (group_box's
// arithmetic on the same minima and maxima), the octree walk (walk_group with the capacities of
// that pass) and, through radius(i), whatever per-target values the stage prepares; the leaves go
// to the pool and the box with the pool position to the group's plan.  Warps share nothing.
template <int D, typename T, class Radius>
__device__ void walk_groups(const GroupWork& work, const TreeView& tv, const Periodic& pb, const State& st,
                            bool use_ksize, const PlanView<T>& pv, int stack_cap, int cap, Radius radius,
                            unsigned char* smem)
{
    using V4 = typename Vec4<T>::type;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned char* base = smem + plan_warp_bytes<T>(stack_cap, cap) * w;
    GroupMisc* gm = reinterpret_cast<GroupMisc*>(base);
    int* stack = reinterpret_cast<int*>(base + align16(sizeof(GroupMisc)));
    int2* leaves = reinterpret_cast<int2*>(base + align16(sizeof(GroupMisc)) + align16(sizeof(int) * (size_t)stack_cap));
    V4* loff = reinterpret_cast<V4*>(base + align16(sizeof(GroupMisc)) + align16(sizeof(int) * (size_t)stack_cap) +
                                     align16(sizeof(int2) * (size_t)cap));
    const long long top = dbl_to_ord(1.7976931348623157e308), bottom = dbl_to_ord(-1.7976931348623157e308);
    for (;;) {
        int k = 0;
        if (lane == 0) k = atomicAdd(work.counter, 1);
        k = __shfl_sync(FULL, k, 0);
        if (k >= *work.n_groups) break;
        const int gb = work.g_begin[k], gn = work.g_count[k];
        if (gn == 0) {
            if (lane == 0 && k < pv.plan_cap) pv.plan[k].nleaves = -2;
            continue;
        }
        long long lo[D], hi[D];
        long long rr = 0, rm = top;
#pragma unroll
        for (int q = 0; q < D; ++q) { lo[q] = top; hi[q] = bottom; }
        for (int q = lane; q < gn; q += 32) {
            const int i = gb + q;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const long long o = dbl_to_ord(st.f[F_POS + d][i]);
                lo[d] = min(lo[d], o);
                hi[d] = max(hi[d], o);
            }
            const long long r = dbl_to_ord(radius(i));
            rr = max(rr, r);
            rm = min(rm, r);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
                lo[d] = min(lo[d], __shfl_xor_sync(FULL, lo[d], o));
                hi[d] = max(hi[d], __shfl_xor_sync(FULL, hi[d], o));
            }
            rr = max(rr, __shfl_xor_sync(FULL, rr, o));
            rm = min(rm, __shfl_xor_sync(FULL, rm, o));
        }
        if (k >= pv.plan_cap) continue;   // no plan: the pair kernel forms the box and walks
        if (lane == 0) {
            double a[3] = {0.0, 0.0, 0.0}, b[3] = {0.0, 0.0, 0.0};
#pragma unroll
            for (int d = 0; d < D; ++d) { a[d] = ord_to_dbl(lo[d]); b[d] = ord_to_dbl(hi[d]); }
            finish_box<D>(gm, a, b, ord_to_dbl(rr), ord_to_dbl(rm), pb);
        }
        __syncwarp();
        const int nl = walk_group<D, T>(tv, st.run[gb], gm, use_ksize, pb, stack, stack_cap, leaves, loff, cap);
        __syncwarp();
        int off = 0;
        if (nl > 0) {
            if (lane == 0) off = atomicAdd(pv.pool_count, nl);
            off = __shfl_sync(FULL, off, 0);
        }
        const bool fits = nl >= 0 && off + nl <= pv.pool_cap;
        if (fits) {
            for (int q = lane; q < nl; q += 32) {
                pv.leaves[off + q] = leaves[q];
                pv.loff[off + q] = loff[q];
            }
        }
        if (lane == 0) {
            GroupPlan* P = pv.plan + k;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                P->gc[d] = gm->gc[d]; P->he[d] = gm->he[d]; P->gcf[d] = gm->gcf[d]; P->hef[d] = gm->hef[d];
            }
            P->R = gm->R; P->rmin = gm->rmin; P->span = gm->span; P->scale = gm->scale; P->bmax = gm->bmax;
            P->Rf = gm->Rf;
            P->nleaves = nl < 0 ? -1 : (fits ? nl : -2);
            P->leaf_off = off;
        }
        __syncwarp();
    }
}

// The plan of the CTA's current group into its shared layout (block-wide): 1 loaded, 0 no plan (box
// and walk in the pair kernel), -1 the planned walk overflowed (the range goes to a later pass).
template <typename T>
__device__ int load_plan(unsigned char* smem, const SmemLayout& L, GroupMisc* gm, const PlanView<T>& pv)
{
    using V4 = typename Vec4<T>::type;
    const int k = gm->gidx;
    if (!pv.plan || k < 0 || k >= pv.plan_cap) return 0;
    const GroupPlan* P = pv.plan + k;
    const int nl = P->nleaves;
    if (nl == -2 || nl > L.leaf_cap) return 0;
    // every thread has taken the range length from gm->ntile (next_group's scratch) before the
    // fields below are overwritten
    __syncthreads();
    if (nl < 0) {
        if (threadIdx.x == 0) { gm->R = P->R; gm->nleaves = 0; gm->overflow = 1; }
        __syncthreads();
        return -1;
    }
    int2* leaves = reinterpret_cast<int2*>(smem + L.off_leaves);
    V4* loff = reinterpret_cast<V4*>(smem + L.off_loff);
    const int off = P->leaf_off;
    for (int q = threadIdx.x; q < nl; q += blockDim.x) {
        leaves[q] = pv.leaves[off + q];
        loff[q] = pv.loff[off + q];
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { gm->gc[d] = P->gc[d]; gm->he[d] = P->he[d]; gm->gcf[d] = P->gcf[d]; gm->hef[d] = P->hef[d]; }
        gm->R = P->R; gm->rmin = P->rmin; gm->span = P->span; gm->scale = P->scale; gm->bmax = P->bmax;
        gm->Rf = P->Rf;
        gm->nleaves = nl;
        gm->ntile = 0;
        gm->overflow = 0;
    }
    __syncthreads();
    return 1;
}

// Per-axis acceptance limit in T for staged offsets: |off_k| <= lim_k keeps every source whose
// exact offset is within ext_k, given the rounding of off (below u (2 |off| + 2 bmax)).
template <typename T>
__device__ __forceinline__ T accept_limit(double ext, const GroupMisc* gm)
{
    const double u = Unit<T>::u;
    return to_T_up<T>(ext * (1.0 + 8.0 * u) + 4.0 * u * gm->bmax + 1e-300);
}

// Rounded-box acceptance for staging: keep a source whose distance from the group's bounding
// box (gc +/- he) is at most r.  Every target lies in the box, so this keeps every source within
// r of some target.  The T offsets differ from the exact ones by at most u (2 |off| + 2 bmax) per
// component; the test shrinks the computed per-axis distances by that bound and widens r, so it
// never drops a source the exact test keeps.
template <int D, typename T>
struct BoxAccept {
    T he[D];
    T slack;
    __device__ __forceinline__ void init(const GroupMisc* gm)
    {
        const double u = Unit<T>::u;
#pragma unroll
        for (int k = 0; k < D; ++k) he[k] = to_T_up<T>(gm->he[k] * (1.0 + 8.0 * u));
        slack = to_T_up<T>(3.0 * u * gm->bmax + 1e-300);
    }
    __device__ __forceinline__ bool operator()(const T* off, T r) const
    {
        const T shrink = T(1) - T(4.0 * Unit<T>::u);
        T d2 = T(0);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const T dk = fabs(off[k]) * shrink - he[k] - slack;
            if (dk > T(0)) d2 += dk * dk;
        }
        const T rr = r * T(1.0 + 8.0 * Unit<T>::u);
        return d2 <= rr * rr;
    }
};

// ---- bulk copies (cp.async.bulk with mbarrier completion) ----------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// Once per CTA, before the first group (block-wide).
__device__ __forceinline__ void bulk_stage_init(GroupMisc* gm)
{
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&gm->mbar)) : "memory");
        gm->mbar_phase = 0u;
    }
    __syncthreads();
}

// Bounded wait for the given phase of the staging mbarrier; false when it ran out.
__device__ __forceinline__ bool bulk_wait(const GroupMisc* gm, unsigned phase, int limit)
{
    const unsigned addr = smem_addr(&gm->mbar);
    for (int it = 0; it < limit; ++it) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(addr), "r"(phase) : "memory");
        if (done) return true;
    }
    return false;
}

// ---- 3. staging -------------------------------------------------------------------------------
// Flattens the leaf ranges and calls, for each particle j (key slot) in deterministic order,
// accept(j, off) with off[k] = (leaf centre - gc) + (x_j - leaf centre) in T; accepted sources
// get consecutive tile slots with their offsets, mass (xrel[j].w) and aux(j).  Returns the tile
// count, or -1 on overflow.
// With bulk (the CTA ran bulk_stage_init) and when all particles of the walked leaves fit the tile,
// the leaves' records are brought into the tile by bulk asynchronous copies (one cp.async.bulk per
// leaf, completion counted on the CTA's mbarrier) and filtered in place, instead of by each thread's
// own loads; the accepted sources, their slots and their order are the same.  A copy wait that
// runs out (bounded twice) raises ERR_TIMEOUT in *err and sends the range to a later pass.
template <int D, typename T, class Accept, class Aux>
__device__ int stage_sources(unsigned char* smem, const SmemLayout& L, GroupMisc* gm,
                             const typename Vec4<T>::type* xrel, const Tile<T>& tile,
                             Accept accept, Aux aux, bool bulk = false, unsigned* err = nullptr)
{
    using V4 = typename Vec4<T>::type;
    int2* leaves = reinterpret_cast<int2*>(smem + L.off_leaves);
    const V4* loff = reinterpret_cast<const V4*>(smem + L.off_loff);
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
    int base = 0;
    const bool in_place = bulk && total <= L.tcap;
    if (in_place) {
        // thread 0 announces the bytes, then warp 0 issues one copy per leaf into the tile at the
        // leaf's prefix position (the tile's earlier readers finished at next_group's barrier)
        const unsigned phase = gm->mbar_phase;
        if (w == 0) {
            if (lane == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                             :: "r"(smem_addr(&gm->mbar)), "r"((unsigned)(total * (int)sizeof(V4))) : "memory");
            }
            __syncwarp();
            for (int l = lane; l < nl; l += 32) {
                const int2 lf = leaves[l];
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                             :: "r"(smem_addr(tile.pm + lpre[l])), "l"(xrel + lf.x),
                                "r"((unsigned)(lf.y * (int)sizeof(V4))), "r"(smem_addr(&gm->mbar))
                             : "memory");
            }
        }
        bool ok = bulk_wait(gm, phase, 1 << 20);
        // the copies are this CTA's own: a second bounded wait before giving the range up
        if (!ok) ok = bulk_wait(gm, phase, 1 << 20);
        if (!ok) {
            if (threadIdx.x == 0 && err) atomicOr(err, (unsigned)ERR_TIMEOUT);
            __syncthreads();
            return -1;
        }
    }
    if (!in_place) {
        // each thread takes a contiguous run of at most 64 flattened positions per chunk (one leaf
        // search per run, then the leaf index only advances), marks the sources it accepts in a
        // bit mask, and writes them after a block-wide scan of the accepted counts: the slots
        // follow f, as in the strided loop below
        const int T_ = blockDim.x;
        for (int c0 = 0; c0 < total; c0 += 64 * T_) {
            const int csz = min(total - c0, 64 * T_);
            const int K = (csz + T_ - 1) / T_;
            const int fb = c0 + min(csz, threadIdx.x * K), fe = c0 + min(csz, threadIdx.x * K + K);
            int l0 = 0;
            if (fb < fe) {
                int hi = nl;   // last leaf with lpre <= fb
                while (hi - l0 > 1) {
                    const int mid = (l0 + hi) >> 1;
                    if (lpre[mid] <= fb) l0 = mid; else hi = mid;
                }
            }
            unsigned long long acc = 0ull;
            {
                int l = l0, lend = lpre[l0 + 1];
                for (int f = fb; f < fe; ++f) {
                    while (f >= lend) { ++l; lend = lpre[l + 1]; }
                    const int j = leaves[l].x + (f - lpre[l]);
                    const V4 a = loff[l];
                    const V4 q = xrel[j];
                    T off[D];
                    off[0] = a.x + q.x;
                    if (D > 1) off[D > 1 ? 1 : 0] = a.y + q.y;
                    if (D > 2) off[D > 2 ? 2 : 0] = a.z + q.z;
                    if (accept(j, off)) acc |= 1ull << (f - fb);
                }
            }
            // block-wide exclusive scan of the accepted counts
            const int cnt = __popcll(acc);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += v;
            }
            __syncthreads();   // earlier readers of wcnt are done
            if (lane == 31) wcnt[w] = incl;
            __syncthreads();
            int woff = 0, tot = 0;
            for (int ww = 0; ww < nw; ++ww) {
                const int v = wcnt[ww];
                if (ww < w) woff += v;
                tot += v;
            }
            int slot = base + woff + incl - cnt;
            if (base + tot <= L.tcap) {
                int l = l0, lend = lpre[l0 + 1];
                while (acc) {
                    const int k = __ffsll((long long)acc) - 1;
                    acc &= acc - 1;
                    const int f = fb + k;
                    while (f >= lend) { ++l; lend = lpre[l + 1]; }
                    const int j = leaves[l].x + (f - lpre[l]);
                    const V4 a = loff[l];
                    const V4 q = xrel[j];
                    V4 v;
                    v.x = a.x + q.x;
                    v.y = D > 1 ? a.y + q.y : T(0);
                    v.z = D > 2 ? a.z + q.z : T(0);
                    v.w = q.w;
                    tile.pm[slot] = v;
                    tile.aux[slot] = aux(j);
                    tile.idx[slot] = j;
                    ++slot;
                }
            }
            base += tot;
            // the range goes to a later pass: no need to count the rest (base is block-uniform)
            if (base > L.tcap) break;
        }
    }
    // (bulk copies in place) U sources per thread between barriers: their loads overlap, and the
    // slot order (by f) is the same as one source per thread per barrier
    constexpr int U = 4;
    for (int f0 = 0; in_place && f0 < total; f0 += U * blockDim.x) {
        bool ok[U];
        int jj[U];
        T off[U][D];
        T mm[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int f = f0 + u * blockDim.x + threadIdx.x;
            ok[u] = false;
            jj[u] = -1;
            mm[u] = T(0);
#pragma unroll
            for (int k = 0; k < D; ++k) off[u][k] = T(0);
            if (f < total) {
                int lo = 0, hi = nl;   // last r with lpre[r] <= f
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (lpre[mid] <= f) lo = mid; else hi = mid;
                }
                const int j = leaves[lo].x + (f - lpre[lo]);
                const V4 a = loff[lo];
                const V4 q = in_place ? tile.pm[f] : xrel[j];
                off[u][0] = a.x + q.x;
                if (D > 1) off[u][D > 1 ? 1 : 0] = a.y + q.y;
                if (D > 2) off[u][D > 2 ? 2 : 0] = a.z + q.z;
                mm[u] = q.w;
                jj[u] = j;
                ok[u] = accept(j, off[u]);
            }
        }
        unsigned bal[U];
#pragma unroll
        for (int u = 0; u < U; ++u) bal[u] = __ballot_sync(FULL, ok[u]);
        __syncthreads();   // previous iteration's readers of wcnt are done
        if (lane == 0) {
#pragma unroll
            for (int u = 0; u < U; ++u) wcnt[u * nw + w] = __popc(bal[u]);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < U; ++u) {
            int woff = 0, tot = 0;
            for (int ww = 0; ww < nw; ++ww) {
                const int c = wcnt[u * nw + ww];
                if (ww < w) woff += c;
                tot += c;
            }
            if (ok[u]) {
                const int slot = base + woff + __popc(bal[u] & lanemask_lt());
                if (slot < L.tcap) {
                    V4 v;
                    v.x = off[u][0];
                    v.y = D > 1 ? off[u][D > 1 ? 1 : 0] : T(0);
                    v.z = D > 2 ? off[u][D > 2 ? 2 : 0] : T(0);
                    v.w = mm[u];
                    tile.pm[slot] = v;
                    tile.aux[slot] = aux(jj[u]);
                    tile.idx[slot] = jj[u];
                }
            }
            base += tot;
        }
        // the range goes to a later pass: no need to count the rest (base is block-uniform)
        if (base > L.tcap) break;
    }
    __syncthreads();
    if (in_place && threadIdx.x == 0) gm->mbar_phase ^= 1u;
    if (base > L.tcap) {
        if (threadIdx.x == 0) gm->overflow = 1000000 + base;   // diagnostic: sources needed (at least)
        return -1;
    }
    // bounding boxes of the mask words (warp w reduces words w, w + nw, ...).  Built in 3D only:
    // a warp skips a word only when none of its 32 targets needs it, which the 2D tiles rarely
    // allow, while in 3D the tile volume outside the targets' spheres is large.
    if (D != 3) return base;
    const T big = sizeof(T) == 4 ? T(3.0e38f) : T(1.0e300);
    for (int wd = w; wd < ((base + 31) >> 5); wd += nw) {
        const int sidx = wd * 32 + lane;
        V4 lo, hi;
        if (sidx < base) {
            lo = tile.pm[sidx];
            lo.w = tile.aux[sidx];
            hi = lo;
        } else {
            lo.x = lo.y = lo.z = lo.w = big;
            hi.x = hi.y = hi.z = hi.w = -big;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo.x = fmin(lo.x, __shfl_xor_sync(FULL, lo.x, o));
            lo.y = fmin(lo.y, __shfl_xor_sync(FULL, lo.y, o));
            lo.z = fmin(lo.z, __shfl_xor_sync(FULL, lo.z, o));
            lo.w = fmin(lo.w, __shfl_xor_sync(FULL, lo.w, o));
            hi.x = fmax(hi.x, __shfl_xor_sync(FULL, hi.x, o));
            hi.y = fmax(hi.y, __shfl_xor_sync(FULL, hi.y, o));
            hi.z = fmax(hi.z, __shfl_xor_sync(FULL, hi.z, o));
            hi.w = fmax(hi.w, __shfl_xor_sync(FULL, hi.w, o));
        }
        if (lane == 0) {
            tile.wbox[2 * wd] = lo;
            tile.wbox[2 * wd + 1] = hi;
        }
    }
    __syncthreads();
    return base;
}

// ---- thread-per-particle walk -----------------------------------------------------------------
// The octree walk of one target on its own (the thread-per-particle schedule): a depth-first walk
// with a per-thread stack that visits the particles of every leaf whose box can lie within the
// reach of x_i per axis (BHTree::neighbor_search, src/bhtree.cpp:239-249; reach = r, or
// max(r, node kernel size) with use_ksize), tested in FP32 on the node mirrors with a relative
// margin and an absolute slack that keep every node the exact FP64 test keeps.  For each leaf the
// offset of its centre from x_i is formed once in FP64 and rounded to T, so a source's separation
// is x_j - x_i = coff + (x_j - leaf centre) with the second term from the per-particle mirror.
constexpr int WALK_STACK = 160;   // 7 waiting siblings per level of a 21-level 3D octree, and more

template <int D, typename T>
struct TargetWalk {
    const TreeView* tv;
    const Periodic* pb;
    double xi[D];
    float xf[D];
    float slack, rf, xmag;
    bool use_ksize;
    bool overflow;
    int sp, jb, je;
    T coff[D];   // leaf centre - x_i
    T bq;        // bound on |x_j - leaf centre| per axis for the current leaf
    T amax;      // max_k |coff_k| + bq of the current leaf
    int* stack;  // WALK_STACK entries owned by the caller (a local array, so that the walker's
                 // scalars can stay in registers)

    __device__ __forceinline__ void start(int* stk, const TreeView& t, const Periodic& p, const double* x, int root,
                                          double r, bool ksize)
    {
        stack = stk;
        tv = &t;
        pb = &p;
        float mag = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            xi[k] = x[k];
            xf[k] = (float)x[k];
            mag = fmaxf(mag, fabsf(xf[k]) + (p.on ? p.lenf[k] : 0.f));
        }
        xmag = mag;
        slack = 4.0f * 5.9604645e-08f * mag + 1e-30f;
        rf = __double2float_ru(r);
        use_ksize = ksize;
        overflow = false;
        stack[0] = root;
        sp = 1;
        jb = je = 0;
    }

    // The next particle (key slot j) of a walked leaf; false when the walk is done.
    __device__ __forceinline__ bool next(int& j)
    {
        while (jb >= je) {
            if (sp == 0) return false;
            const int node = stack[--sp];
            if (tv->count[node] <= 0) continue;
            const float e2 = 0.5f * tv->ef[node];
            const float reach = use_ksize ? fmaxf(rf, tv->kf[node]) : rf;
            bool hit = true;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const float d = fabsf(min_image_f(tv->cf[k][node] - xf[k], *pb, k));
                if (d > (e2 + reach) * 1.00001f + slack) hit = false;
            }
            if (!hit) continue;
            const int fc = tv->first_child[node];
            if (fc < 0) {
                jb = tv->begin[node];
                je = jb + tv->count[node];
                T am = T(0);
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    coff[k] = (T)min_image(tv->center[k][node] - xi[k], *pb, k);
                    am = fmax(am, fabs(coff[k]));
                }
                bq = (T)(0.5 * tv->edge[node] * (1.0 + 1e-6));
                amax = am + bq;
            } else {
                const int nc = tv->nchild[node];
                if (sp + nc > WALK_STACK) { overflow = true; sp = 0; jb = je = 0; return false; }
                for (int c = nc - 1; c >= 0; --c) stack[sp++] = fc + c;
            }
        }
        j = jb++;
        return true;
    }

    // Separation x_i - x_j in T of slot j of the current leaf (q = its {x_j - leaf centre, m}) and
    // the bound on the rounding error of r^2 = |x_i - x_j|^2 for separations up to rmax.
    template <class V4>
    __device__ __forceinline__ T sep(const V4& q, T* rv) const
    {
        rv[0] = -(coff[0] + q.x);
        T r2 = rv[0] * rv[0];
        if (D > 1) { rv[D > 1 ? 1 : 0] = -(coff[D > 1 ? 1 : 0] + q.y); r2 = fma(rv[D > 1 ? 1 : 0], rv[D > 1 ? 1 : 0], r2); }
        if (D > 2) { rv[D > 2 ? 2 : 0] = -(coff[D > 2 ? 2 : 0] + q.z); r2 = fma(rv[D > 2 ? 2 : 0], rv[D > 2 ? 2 : 0], r2); }
        return r2;
    }
    __device__ __forceinline__ T band(T rmax) const
    {
        // per component: rounding of coff and of the sum, below 2 u (|coff| + bq), plus the FP64
        // rounding of the centre offset against the coordinate scale
        const T u = T(Unit<T>::u);
        const T E = T(2.5) * u * amax + T(8.0 * Unit<double>::u) * (amax + T(xmag));
        return T(2.0 * 1.7320508075688772) * E * rmax + T(D) * E * E + T(D + 3) * u * rmax * rmax;
    }
};

// ---- exact FP64 decisions for the guard band ---------------------------------------------------
template <int D>
__device__ __forceinline__ double exact_r2(const State& st, const double* xi, int j, const Periodic& pb)
{
    double xj[D];
#pragma unroll
    for (int k = 0; k < D; ++k) xj[k] = st.f[F_POS + k][j];
    return ref_r2<D>(xi, xj, pb);
}

// Bound on the rounding error of each component of a T-precision separation between a target
// (|xo| <= he) and a staged source (|p| <= span), for separations up to h:
// E = u (he + 2 |p| + 2 bmax + |r|) <= u (3 span + 2 bmax + h), plus the FP64 rounding of the
// offsets against the coordinate scale.
template <typename T>
__device__ __forceinline__ double comp_err(const GroupMisc* gm, double h)
{
    const double u = Unit<T>::u;
    return u * (3.0 * gm->span + 2.0 * gm->bmax + h) * 1.25 + 8.0 * Unit<double>::u * (gm->span + h + gm->scale);
}

// Guard band of |r2_T - r2_exact| for pairs with separation <= h.
template <typename T, int D>
__device__ __forceinline__ double r2_band(const GroupMisc* gm, double h)
{
    const double u = Unit<T>::u;
    const double E = comp_err<T>(gm, h);
    return 2.0 * 1.7320508075688772 * E * h + D * E * E + (D + 2) * u * h * h;
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
