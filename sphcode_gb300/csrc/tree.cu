// Octree construction on the device (replaces BHTree::make / create_tree / assign,
// src/bhtree.cpp:55-107,136-204, and BHTree::set_kernel, :109-112,206-232).
//
// The reference splits a node at its geometric center with `pos > center` per axis and builds
// children's centers as center +/- edge/4 (src/bhtree.cpp:170-175,190-196).  Every particle's
// path through that recursion is its key: per level, the D comparison bits against the FP64
// center sequence the reference would compute.  Sorting by those keys (radix sort) puts each
// node's particles in one contiguous range, so nodes are built level by level as ranges, with
// the reference's split rule (num > leafParticleNumber and level <= maxTreeLevel; the root always
// splits) and its node-pool capacity of 5 N.  Node mass, centre of mass and kernel size are
// reduced bottom-up.  The roots' mass and centre of mass stay zero, as in the reference, whose
// root never receives them (include/bhtree.hpp:46-53, src/bhtree.cpp:57).
#include "context.cuh"

namespace sphgpu {

namespace {

constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ITEMS = 16;
constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ITEMS;
constexpr int LEVEL_CHUNK = 1024;

// ---- root boxes ---------------------------------------------------------------------------

__global__ void bbox_init_kernel(long long* bbox, int R, int D)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R * D) return;
    const int r = i / D, k = i % D;
    bbox[r * 2 * D + k] = dbl_to_ord(1.7976931348623157e308);
    bbox[r * 2 * D + D + k] = dbl_to_ord(-1.7976931348623157e308);
}

// Bounding box of every run on the ordered-integer images of the coordinates (min / max of the
// images are those of the doubles).  Each warp takes BBOX_ROWS coalesced rows of 32 particles and
// keeps per-lane extremes while its run stays the same (runs are contiguous), so a run issues
// about one atomic per warp and axis instead of one per 32 particles.
constexpr int BBOX_ROWS = 16;
template <int D>
__global__ void bbox_kernel(State st, int n, long long* bbox)
{
    const int lane = threadIdx.x & 31;
    const long long base = (long long)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 * BBOX_ROWS;
    const long long EMPTY_LO = dbl_to_ord(1.7976931348623157e308), EMPTY_HI = dbl_to_ord(-1.7976931348623157e308);
    long long lo[D], hi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { lo[k] = EMPTY_LO; hi[k] = EMPTY_HI; }
    int cur = -1;
    auto flush = [&](int r) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            atomicMin(&bbox[r * 2 * D + k], lo[k]);
            atomicMax(&bbox[r * 2 * D + D + k], hi[k]);
            lo[k] = EMPTY_LO;
            hi[k] = EMPTY_HI;
        }
    };
    for (int q = 0; q < BBOX_ROWS; ++q) {
        const long long i = base + q * 32 + lane;
        if (i >= n) break;
        const int r = st.run[i];
        if (r != cur) {
            if (cur >= 0) flush(cur);
            cur = r;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const long long b = __double_as_longlong(st.f[F_POS + k][i]);
            if ((b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) continue;   // NaN: left out, as fmin/fmax do
            const long long o = b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
            lo[k] = o < lo[k] ? o : lo[k];
            hi[k] = o > hi[k] ? o : hi[k];
        }
    }
    // lanes that end in the same run combine before the atomics
    const unsigned same = __match_any_sync(FULL, cur);
    if (same == FULL) {
        if (cur < 0) return;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            for (int o = 16; o > 0; o >>= 1) {
                const long long a = __shfl_xor_sync(FULL, lo[k], o), b = __shfl_xor_sync(FULL, hi[k], o);
                lo[k] = a < lo[k] ? a : lo[k];
                hi[k] = b > hi[k] ? b : hi[k];
            }
        }
        if (lane == 0) flush(cur);
    } else if (cur >= 0) {
        flush(cur);
    }
}

// Root node of every run (BHTree::initialize / BHTree::make, src/bhtree.cpp:12-40,59-95):
// periodic -> center of the range, edge = largest range; else the bounding box of the run.
template <int D>
__global__ void roots_kernel(TreeView tv, double* center0, double* center1, double* center2,
                             double* edge, int* begin, int* count, int* first, int* nchild,
                             int* level, int* parent, int* arrive, double* mass, double* com0,
                             double* com1, double* com2, const long long* bbox,
                             const int* run_begin, int R, Periodic pb, int* lvl_start)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) { lvl_start[0] = 0; lvl_start[1] = 0; lvl_start[2] = R; }
    if (r >= R) return;
    double* cen[3] = {center0, center1, center2};
    double l = 0.0;
    for (int k = 0; k < D; ++k) {
        double lo, hi;
        if (pb.on) { lo = pb.lo[k]; hi = pb.hi[k]; }
        else { lo = ord_to_dbl(bbox[r * 2 * D + k]); hi = ord_to_dbl(bbox[r * 2 * D + D + k]); }
        cen[k][r] = (hi + lo) * 0.5;
        const double range = hi - lo;
        if (l < range) l = range;
    }
    edge[r] = l;
    begin[r] = run_begin[r];
    count[r] = run_begin[r + 1] - run_begin[r];
    first[r] = -1;
    nchild[r] = 0;
    level[r] = 1;
    parent[r] = -1;
    arrive[r] = 0;
    mass[r] = 0.0;
    com0[r] = 0.0;
    if (com1) com1[r] = 0.0;
    if (com2) com2[r] = 0.0;
}

// ---- keys -------------------------------------------------------------------------------

// Centres of the first KEY_TABLE_LEVELS levels of every run's split, per axis: the centre
// recursion of keys_kernel replayed once per node of a complete binary tree (heap order: node k
// has children 2k (x <= c) and 2k + 1 (x > c)), with the same FP64 operations in the same order,
// so a particle's path through the table equals its path through the recursion.  Entries
// k < 2^T hold the ordered-integer image of the centre (compared against), entries 2^T <= k < 2^(T+1)
// the centre itself (where the particle's recursion continues).
// T is chosen at creation: the most levels, up to KEY_TABLE_LEVELS, whose tables of all runs fit
// KEY_TABLE_BYTES (a single run takes ten levels; a batch of 4096 1D runs eight).
constexpr int KEY_TABLE_LEVELS = 10;
constexpr size_t KEY_TABLE_BYTES = 64u << 20;

__global__ void key_table_kernel(TreeView tv, int R, int D, int T, long long* table)
{
    const int ts = 2 << T;
    const long long total = (long long)R * D * ts;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q % ts);
        const int ax = (int)((q / ts) % D);
        const int r = (int)(q / ((long long)ts * D));
        if (k == 0) { table[q] = 0; continue; }
        const int depth = 31 - __clz(k);
        double c = tv.center[ax][r] + 0.0;
        const double e0 = tv.edge[r];
        const bool scale = e0 > 0.0;
        long long qb = scale ? __double_as_longlong(e0) - (2LL << 52) : 0;
        for (int l = 0; l < depth; ++l) {
            const double qd = scale ? __longlong_as_double(qb) : 0.0;
            const bool up = (k >> (depth - 1 - l)) & 1;
            c = __dadd_rn(c, up ? qd : -qd);
            qb -= 1LL << 52;
        }
        table[q] = depth < T ? dbl_to_ord(c) : __double_as_longlong(c);
    }
}

// The path of a particle through the reference's recursive split, one D-bit digit per level,
// most significant first, with the run index above the digits.  With a table (T > 0) the first
// T levels are a search through it (integer comparisons, no FP64 arithmetic) and the recursion
// continues from the level-T centre the search ends at.
template <int D>
__global__ void keys_kernel(State st, int n, TreeView tv, int levels, int nd, int run_shift,
                            unsigned long long* keys, int* perm, const long long* table, int T)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = st.run[i];
    double x[D], c[D];
#pragma unroll
    // + 0.0 turns -0.0 into +0.0, so that the ordered-integer comparison below equals x > c
    for (int k = 0; k < D; ++k) { x[k] = st.f[F_POS + k][i] + 0.0; c[k] = tv.center[k][r] + 0.0; }
    // edge / 4 of level l is the root edge scaled by 2^-(l+2): exact, so it is formed on the
    // exponent bits; only the centre update needs FP64 arithmetic, and the comparison x > c runs on
    // the ordered-integer images of the doubles
    const double e0 = tv.edge[r];
    const bool scale = e0 > 0.0;   // a zero-extent root keeps every centre (edge * 0.25 = 0)
    long long q = scale ? __double_as_longlong(e0) - (2LL << 52) : 0;
    long long xo[D];
#pragma unroll
    for (int k = 0; k < D; ++k) xo[k] = dbl_to_ord(x[k]);
    unsigned long long key = 0;
    int l0 = 0;
    if (T > 0) {
        const int ts = 2 << T;
        const long long* tb = table + (size_t)r * D * ts;
        int kk[D];
#pragma unroll
        for (int k = 0; k < D; ++k) kk[k] = 1;
        for (int l = 0; l < T; ++l) {
            unsigned digit = 0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const bool up = xo[k] > __ldg(tb + k * ts + kk[k]);
                digit |= (up ? 1u : 0u) << k;
                kk[k] = 2 * kk[k] + (up ? 1 : 0);
            }
            key = (key << D) | digit;
        }
#pragma unroll
        for (int k = 0; k < D; ++k) c[k] = __longlong_as_double(__ldg(tb + k * ts + kk[k]));
        q -= (long long)T << 52;
        l0 = T;
    }
    // the first nd digits (the levels a capped build splits); deeper digits stay 0
    for (int l = l0; l < nd; ++l) {
        unsigned digit = 0;
        const double qd = scale ? __longlong_as_double(q) : 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const bool up = xo[k] > dbl_to_ord(c[k]);
            digit |= (up ? 1u : 0u) << k;
            // child center: center + (+/-1 * edge) * 0.25, one rounding (src/bhtree.cpp:190-196)
            c[k] = __dadd_rn(c[k], up ? qd : -qd);
        }
        key = (key << D) | digit;
        q -= 1LL << 52;
    }
    if (nd < levels) key <<= D * (levels - nd);
    if (run_shift < 64) key |= (unsigned long long)r << run_shift;
    keys[i] = key;
    perm[i] = i;
}

// ---- radix sort (LSD, 8-bit digits, stable) ---------------------------------------------

__global__ void radix_hist_kernel(const unsigned long long* keys, int n, int shift, int* hist,
                                  int nblocks)
{
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RADIX_TILE;
    for (int i = threadIdx.x; i < RADIX_TILE; i += RADIX_THREADS) {
        const int idx = base + i;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of each digit's column of per-block counts (hist[d * nblocks + b]), one block per
// digit; the digit totals go to dtot.
__global__ void radix_scan_columns_kernel(int* hist, int nblocks, int* dtot)
{
    __shared__ int part[32];
    int* col = hist + (size_t)blockIdx.x * nblocks;
    const int t = threadIdx.x;
    const int per = (nblocks + 1023) / 1024;
    const int b = t * per, e = min(nblocks, b + per);
    int sum = 0;
    for (int i = b; i < e; ++i) sum += col[i];
    // block scan of the 1024 partial sums: warp scans, then a scan of the 32 warp totals
    const int lane = t & 31, w = t >> 5;
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) part[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = part[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        part[lane] = x;
    }
    __syncthreads();
    incl += w > 0 ? part[w - 1] : 0;
    int run = incl - sum;
    for (int i = b; i < e; ++i) {
        const int v = col[i];
        col[i] = run;
        run += v;
    }
    if (t == 1023) dtot[blockIdx.x] = incl;
}

__global__ void radix_scatter_kernel(const unsigned long long* kin, const int* vin,
                                     unsigned long long* kout, int* vout, int n, int shift,
                                     const int* hist, int nblocks, const int* dtot)
{
    __shared__ int base[256];
    __shared__ int wcnt[RADIX_THREADS / 32][256];
    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    // digit offset = sum of the totals of the smaller digits (block scan of dtot)
    base[t] = dtot[t];
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const int v = t >= o ? base[t - o] : 0;
        __syncthreads();
        base[t] += v;
        __syncthreads();
    }
    const int excl = base[t] - dtot[t];
    __syncthreads();
    base[t] = excl + hist[t * nblocks + blockIdx.x];
    // the tile's keys and values in registers first: one load latency for the tile, not one per round
    unsigned long long kr[RADIX_ITEMS];
    int vr[RADIX_ITEMS];
#pragma unroll
    for (int round = 0; round < RADIX_ITEMS; ++round) {
        const int idx = blockIdx.x * RADIX_TILE + round * RADIX_THREADS + t;
        kr[round] = idx < n ? kin[idx] : 0ull;
        vr[round] = idx < n ? vin[idx] : 0;
    }
#pragma unroll
    for (int round = 0; round < RADIX_ITEMS; ++round) {
        const int idx = blockIdx.x * RADIX_TILE + round * RADIX_THREADS + t;
        const bool valid = idx < n;
        const unsigned long long k = kr[round];
        const int d = valid ? (int)((k >> shift) & 255) : 256;
#pragma unroll
        for (int ww = 0; ww < RADIX_THREADS / 32; ++ww) wcnt[ww][t] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(FULL, d);
        const int rank = __popc(peers & lanemask_lt());
        if (valid && (__ffs(peers) - 1) == lane) wcnt[w][d] = __popc(peers);
        __syncthreads();
        int s = 0;
#pragma unroll
        for (int ww = 0; ww < RADIX_THREADS / 32; ++ww) {
            const int c = wcnt[ww][t];
            wcnt[ww][t] = s;
            s += c;
        }
        __syncthreads();
        if (valid) {
            const int pos = base[d] + wcnt[w][d] + rank;
            kout[pos] = k;
            vout[pos] = vr[round];
        }
        __syncthreads();
        base[t] += s;
    }
}

// ---- reorder ----------------------------------------------------------------------------

struct FieldMove {
    const double* src[F_COUNT];
    double* dst[F_COUNT];
    int nf;
    const int* isrc[2];
    int* idst[2];
    int ni;
};

__global__ void reorder_kernel(FieldMove fm, const int* perm, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = perm[i];
    for (int f = 0; f < fm.nf; ++f) fm.dst[f][i] = fm.src[f][j];
    for (int f = 0; f < fm.ni; ++f) fm.idst[f][i] = fm.isrc[f][j];
}

__global__ void copy_fields_kernel(FieldMove fm, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int f = 0; f < fm.nf; ++f) fm.dst[f][i] = fm.src[f][i];
    for (int f = 0; f < fm.ni; ++f) fm.idst[f][i] = fm.isrc[f][i];
}

// ---- level-by-level node construction ---------------------------------------------------

struct NodeArrays {
    int *begin, *count, *first, *nchild, *parent, *level, *arrive;
    double *center[3], *edge;
    int* bnd;   // per split node, its 2^D - 1 inner child boundaries (found once, used by the next level)
};

template <int D>
__device__ __forceinline__ void child_bounds(const unsigned long long* keys, int b, int cnt,
                                             int shift, int* bnd)
{
    constexpr int NC = 1 << D;
    bnd[0] = b;
    bnd[NC] = b + cnt;
    for (int c = 1; c < NC; ++c) {
        int lo = bnd[c - 1], hi = b + cnt;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const int dg = (int)((keys[mid] >> shift) & (NC - 1));
            if (dg < c) lo = mid + 1; else hi = mid;
        }
        bnd[c] = lo;
    }
}

// child_bounds of one range by the whole warp (b, cnt and the result are the same in every
// lane): 32 probes per round narrow each boundary 32-fold, so a range of 2^20 particles takes
// four rounds of loads per boundary instead of twenty dependent ones.
template <int D>
__device__ __forceinline__ void warp_child_bounds(const unsigned long long* keys, int b, int cnt,
                                                  int shift, int* bnd)
{
    constexpr int NC = 1 << D;
    const int lane = threadIdx.x & 31;
    bnd[0] = b;
    bnd[NC] = b + cnt;
    int lo = b;
#pragma unroll
    for (int c = 1; c < NC; ++c) {
        int hi = b + cnt;   // first index in [lo, hi) with digit >= c, or hi
        while (hi - lo > 32) {
            const int step = (hi - lo + 31) >> 5;
            const int pos = lo + lane * step;
            const bool ge = pos >= hi || (int)((keys[pos] >> shift) & (NC - 1)) >= c;
            const unsigned m = __ballot_sync(FULL, ge);
            if (m == 0) {
                lo = lo + 31 * step + 1;
            } else {
                const int f = __ffs(m) - 1;
                if (f == 0) { hi = lo; break; }
                const int pf = lo + f * step;
                lo = lo + (f - 1) * step + 1;
                hi = pf < hi ? pf : hi;
            }
        }
        if (hi > lo) {
            const int pos = lo + lane;
            const bool ge = pos >= hi || (int)((keys[pos] >> shift) & (NC - 1)) >= c;
            const unsigned m = __ballot_sync(FULL, ge);
            lo = m ? lo + __ffs(m) - 1 : hi;
        }
        bnd[c] = lo;
    }
}

// Child boundaries for every lane with want set (warp-collective: all 32 lanes call it).  A warp
// with one or two large ranges searches them together; otherwise each lane searches its own.
constexpr int WARP_SEARCH_MIN = 4096;
template <int D>
__device__ __forceinline__ void find_bounds(const unsigned long long* keys, bool want, int b, int cnt,
                                            int shift, int* bnd)
{
    constexpr int NC = 1 << D;
    const int lane = threadIdx.x & 31;
    const bool big = want && cnt > WARP_SEARCH_MIN;
    const unsigned bm = __ballot_sync(FULL, big);
    const bool coop = bm != 0 && __popc(bm) <= 2;
    if (want && !(coop && big)) child_bounds<D>(keys, b, cnt, shift, bnd);
    __syncwarp();
    if (coop) {
        unsigned mm = bm;
        while (mm) {
            const int src = __ffs(mm) - 1;
            mm &= mm - 1;
            int wb[NC + 1];
            warp_child_bounds<D>(keys, __shfl_sync(FULL, b, src), __shfl_sync(FULL, cnt, src), shift, wb);
            if (lane == src) {
#pragma unroll
                for (int c = 0; c <= NC; ++c) bnd[c] = wb[c];
            }
        }
    }
}

// First index in [lo, hi) whose level digit (the D bits at shift) is >= c, or hi, searched by a
// group of G lanes (G a power of two from 4 to 32; gl the lane's index in the group, gmask the
// group's lanes in the warp, gshift the group's first lane): each round probes G evenly spaced keys
// and keeps the interval between the last probe below c and the first at or above it, so a range
// of 2^14 particles takes two to four dependent rounds instead of fourteen.
template <int D>
__device__ __forceinline__ int group_first_ge(const unsigned long long* keys, int lo, int hi, int shift, int c,
                                              int G, int gl, unsigned gmask, int gshift)
{
    constexpr int NC = 1 << D;
    const unsigned gbits = G == 32 ? FULL : ((1u << G) - 1u);
    while (hi - lo > G) {
        const int step = (hi - lo + G - 1) / G;
        const int pos = lo + gl * step;
        const bool ge = pos >= hi || (int)((keys[pos] >> shift) & (NC - 1)) >= c;
        const unsigned m = (__ballot_sync(gmask, ge) >> gshift) & gbits;
        if (m == 0) {
            lo = lo + (G - 1) * step + 1;
        } else {
            const int f = __ffs(m) - 1;
            if (f == 0) return lo;
            const int pf = lo + f * step;
            lo = lo + (f - 1) * step + 1;
            hi = pf < hi ? pf : hi;
        }
    }
    if (hi > lo) {
        const int pos = lo + gl;
        const bool ge = pos >= hi || (int)((keys[pos] >> shift) & (NC - 1)) >= c;
        const unsigned m = (__ballot_sync(gmask, ge) >> gshift) & gbits;
        lo = m ? lo + __ffs(m) - 1 : hi;
    }
    return lo;
}

// Counting for a level with few nodes (the upper levels): one task per (node, inner child
// boundary), each searched by a group of G lanes, with G the largest power of two (at most 32,
// at least 4) for which every task has its own group in the grid.  The last task of a node to
// finish (counted on the node's arrival counter, which returns to zero) forms the child count
// from the boundaries the other groups stored.  Returns false, with nothing done, when the level
// has too many nodes for groups of four lanes; every thread of the grid takes the same branch.
template <int D, int NT>
__device__ __forceinline__ bool count_level_grouped(const NodeArrays& na, const unsigned long long* keys, int n,
                                                    int s, int e, int l, int levels, int lv, int leaf_num,
                                                    int* lvl_tmp, int* chunk_sum, int* trunc)
{
    constexpr int NC = 1 << D;
    const long long tasks = (long long)(e - s) * (NC - 1);
    const long long lanes = (long long)gridDim.x * NT;
    int G = 32;
    while (G >= 4 && tasks * G > lanes) G >>= 1;
    if (G < 4) return false;
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), gshift = lane & ~(G - 1);
    const unsigned gmask = (G == 32 ? FULL : ((1u << G) - 1u)) << gshift;
    const long long ngroups = lanes / G;
    const int shift = D * (levels - l);
    for (long long q = ((long long)blockIdx.x * NT + threadIdx.x) / G; q < tasks; q += ngroups) {
        const int node = s + (int)(q / (NC - 1));
        const int c = 1 + (int)(q % (NC - 1));
        int b = __ldcg(na.begin + node), cnt = __ldcg(na.count + node);
        if (b < 0 || cnt < 0 || b + cnt > n) { b = 0; cnt = 0; }
        const bool split = (l == 1) || (cnt > leaf_num && l <= lv);
        if (!split || cnt == 0) {
            if (c == 1 && gl == 0) {
                if (!split && cnt > leaf_num && l <= levels) atomicOr(trunc, 1);
                if (!split) { na.first[node] = -1; na.nchild[node] = 0; }
                lvl_tmp[node - s] = 0;
            }
            continue;
        }
        const int pos = group_first_ge<D>(keys, b, b + cnt, shift, c, G, gl, gmask, gshift);
        if (gl == 0) {
            int* slot = na.bnd + (size_t)node * (NC - 1);
            slot[c - 1] = pos;
            __threadfence();
            if (atomicAdd(na.arrive + node, 1) == NC - 2) {
                __threadfence();
                int prev = b, nc = 0;
                for (int k = 1; k < NC; ++k) {
                    const int x = k == c ? pos : __ldcg(slot + (k - 1));
                    nc += x > prev;
                    prev = x;
                }
                nc += b + cnt > prev;
                lvl_tmp[node - s] = nc;
                atomicAdd(&chunk_sum[(node - s) / LEVEL_CHUNK], nc);
                na.arrive[node] = 0;
            }
        }
    }
    return true;
}

// First index in [lo, hi) whose level digit is >= c, or hi: one thread's binary search.
template <int D>
__device__ __forceinline__ int first_ge(const unsigned long long* keys, int lo, int hi, int shift, int c)
{
    constexpr int NC = 1 << D;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int)((keys[mid] >> shift) & (NC - 1)) < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Counting of the nodes [lo_node, hi_node) of level l by the threads of one block (the nodes this
// block has just placed): one task per (node, inner child boundary), each searched by a group of
// G lanes (G a power of two up to 32, the largest that gives every task its own group in the
// block; a thread per task below two lanes).  Split decision, boundaries, child counts and
// per-chunk totals are those of count_level; the last task of a node forms its child count.
template <int D>
__device__ __forceinline__ void count_nodes_block(const NodeArrays& na, const unsigned long long* keys, int n,
                                                  int lo_node, int hi_node, int s, int l, int levels, int lv,
                                                  int leaf_num, int* lvl_tmp, int* chunk_sum, int* trunc)
{
    constexpr int NC = 1 << D;
    const int tasks = (hi_node - lo_node) * (NC - 1);
    if (tasks <= 0) return;
    int G = 32;
    while (G >= 2 && tasks * G > (int)blockDim.x) G >>= 1;
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), gshift = lane & ~(G - 1);
    const unsigned gmask = (G == 32 ? FULL : ((1u << G) - 1u)) << gshift;
    const int ngroups = (int)blockDim.x / G;
    const int shift = D * (levels - l);
    for (int q = (int)threadIdx.x / G; q < tasks; q += ngroups) {
        const int node = lo_node + q / (NC - 1);
        const int c = 1 + q % (NC - 1);
        int b = __ldcg(na.begin + node), cnt = __ldcg(na.count + node);
        if (b < 0 || cnt < 0 || b + cnt > n) { b = 0; cnt = 0; }
        const bool split = cnt > leaf_num && l <= lv;
        if (!split || cnt == 0) {
            if (c == 1 && gl == 0) {
                if (!split && cnt > leaf_num && l <= levels) atomicOr(trunc, 1);
                if (!split) { na.first[node] = -1; na.nchild[node] = 0; }
                lvl_tmp[node - s] = 0;
            }
            continue;
        }
        const int pos = G >= 2 ? group_first_ge<D>(keys, b, b + cnt, shift, c, G, gl, gmask, gshift)
                               : first_ge<D>(keys, b, b + cnt, shift, c);
        if (gl == 0) na.bnd[(size_t)node * (NC - 1) + (c - 1)] = pos;
    }
    // every task of these nodes ran in this block: after the barrier each node's boundaries are
    // visible to all its threads, and the child counts follow without fences or arrival counters
    __syncthreads();
    const int lane32 = threadIdx.x & 31;
    for (int nb = lo_node; nb < hi_node; nb += blockDim.x) {
        const int node = nb + (int)threadIdx.x;
        int nc = 0;
        if (node < hi_node) {
            int b = __ldcg(na.begin + node), cnt = __ldcg(na.count + node);
            if (b < 0 || cnt < 0 || b + cnt > n) { b = 0; cnt = 0; }
            if (cnt > leaf_num && l <= lv) {
                const int* slot = na.bnd + (size_t)node * (NC - 1);
                int prev = b;
                for (int k = 1; k < NC; ++k) {
                    const int x = slot[k - 1];
                    nc += x > prev;
                    prev = x;
                }
                nc += b + cnt > prev;
                lvl_tmp[node - s] = nc;
            }
        }
        // one add per chunk and warp: a warp's 32 consecutive nodes lie in at most two chunks
        const int chunk = node < hi_node ? (node - s) / LEVEL_CHUNK : -1;
        const int first = __shfl_sync(FULL, chunk, 0);
        const int in_first = __reduce_add_sync(FULL, chunk == first ? nc : 0);
        const int in_second = __reduce_add_sync(FULL, chunk != first ? nc : 0);
        const unsigned second = __ballot_sync(FULL, chunk >= 0 && chunk != first);
        if (lane32 == 0 && first >= 0 && in_first) atomicAdd(&chunk_sum[first], in_first);
        if (second && lane32 == __ffs(second) - 1 && in_second) atomicAdd(&chunk_sum[chunk], in_second);
    }
}

template <int D>
__device__ __forceinline__ void store_bounds(int* buf, int node, const int* bnd)
{
    constexpr int NC = 1 << D;
#pragma unroll
    for (int c = 1; c < NC; ++c) buf[(size_t)node * (NC - 1) + (c - 1)] = bnd[c];
}

constexpr int COUNT_THREADS = 256;
template <int D, int NT>
__device__ __forceinline__ void count_level(const NodeArrays& na, const unsigned long long* keys, int n,
                                            const int* lvl_start, int l, int levels, int lv, int leaf_num,
                                            int* lvl_tmp, int* chunk_sum, int* trunc, int* red)
{
    constexpr int NC = 1 << D;
    // loads of data another block may have written earlier in the same launch go to L2 (__ldcg):
    // the fused build reads, after a grid barrier, what other SMs wrote before it
    const int s = __ldcg(lvl_start + l), e = __ldcg(lvl_start + l + 1);
    if (count_level_grouped<D, NT>(na, keys, n, s, e, l, levels, lv, leaf_num, lvl_tmp, chunk_sum, trunc)) return;
    const int nsub = (e - s + NT - 1) / NT;
    const int spread = (threadIdx.x & 31) * (NT / 32) + (threadIdx.x >> 5);
    for (int sub = blockIdx.x; sub < nsub; sub += gridDim.x) {
        const int node = s + sub * NT + spread;
        int nc = 0;
        bool split = false;
        int b = 0, cnt = 0;
        if (node < e) {
            b = __ldcg(na.begin + node);
            cnt = __ldcg(na.count + node);
            // slots of a parent the node pool could not hold were not written (the error bit is set)
            if (b < 0 || cnt < 0 || b + cnt > n) { b = 0; cnt = 0; }
            split = (l == 1) || (cnt > leaf_num && l <= lv);
            // a node the full build would split, left a leaf by the cap
            if (!split && cnt > leaf_num && l <= levels) atomicOr(trunc, 1);
        }
        int bnd[NC + 1];
        find_bounds<D>(keys, split && cnt > 0, b, cnt, D * (levels - l), bnd);
        if (node < e) {
            if (split && cnt > 0) {
#pragma unroll
                for (int c = 0; c < NC; ++c) nc += bnd[c + 1] > bnd[c];
                store_bounds<D>(na.bnd, node, bnd);
            }
            if (!split) { na.first[node] = -1; na.nchild[node] = 0; }
            lvl_tmp[node - s] = nc;
        }
        // block sum into the chunk's total (a sub-chunk lies within one chunk)
        int v = nc;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x < 32) {
            int u = threadIdx.x < NT / 32 ? red[threadIdx.x] : 0;
            for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(FULL, u, o);
            if (threadIdx.x == 0 && u) atomicAdd(&chunk_sum[(sub * NT) / LEVEL_CHUNK], u);
        }
        __syncthreads();
    }
}

// Split decision (src/bhtree.cpp:154-158), child boundaries and child count of every level-l node,
// with the per-chunk (LEVEL_CHUNK nodes) totals accumulated into chunk_sum (zeroed beforehand).
// Blocks of COUNT_THREADS threads take sub-chunks of as many nodes, spread over the block's warps
// (the first nodes to lane 0 of each warp), so that the few large ranges of the upper levels are
// searched by separate warps.
template <int D>
__global__ void __launch_bounds__(COUNT_THREADS) level_count_kernel(NodeArrays na, const unsigned long long* keys,
                                   int n, const int* lvl_start, int l, int levels, int lv, int leaf_num,
                                   int* lvl_tmp, int* chunk_sum, int* trunc)
{
    __shared__ int red[COUNT_THREADS / 32];
    count_level<D, COUNT_THREADS>(na, keys, n, lvl_start, l, levels, lv, leaf_num, lvl_tmp, chunk_sum, trunc, red);
}


// Places the children of the level-l nodes (level l + 1: begin, count, centre, edge, parent) from
// the child counts and boundaries that the count of level l found (one launch per level, or one
// phase of the fused build).  tmp_cur / cs_cur hold the child counts of the level-l nodes and their
// per-chunk totals (cs_off, when given, their exclusive scan); the call also clears cs_clear, the
// totals that the count of level l + 2 fills.  Node indices are breadth-first and, within a level,
// in key order.  With COUNT, each block also counts the children it has just placed
// (count_nodes_block: split decision, boundaries, child counts into nx.lvl_tmp and nx.chunk_sum),
// so that the fused build needs one grid barrier per level.
struct NextCount {
    const unsigned long long* keys;
    int n, levels, lv, leaf_num;
    int* lvl_tmp;
    int* chunk_sum;
    int* trunc;
};

template <int D, bool COUNT>
__device__ __forceinline__ void build_level(const NodeArrays& na, int* lvl_start, int l, const int* tmp_cur,
                                            const int* cs_cur, int* cs_clear, int cs_cap, int node_cap,
                                            unsigned* err, int* sc, int* red, const NextCount& nx,
                                            const int* cs_off = nullptr)
{
    constexpr int NC = 1 << D;
    static_assert(LEVEL_CHUNK == 1024, "the chunk scan takes 32 warps of 32 nodes");
    const int s = __ldcg(lvl_start + l), e = __ldcg(lvl_start + l + 1);
    const int nchunks = (e - s + LEVEL_CHUNK - 1) / LEVEL_CHUNK;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cs_cap; q += gridDim.x * blockDim.x) cs_clear[q] = 0;
    // block sum of cs_cur[0, m)
    // with cs_off (the chunk totals' exclusive scan, formed by chunk_offsets_kernel) one load;
    // otherwise a block sum, which is O(chunks) per chunk and pays only for levels of few chunks
    auto prefix = [&](int m) {
        if (cs_off) return __ldcg(cs_off + m);
        int v = 0;
        for (int q = threadIdx.x; q < m; q += blockDim.x) v += __ldcg(cs_cur + q);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        int u = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) u += red[w];
        __syncthreads();
        return u;
    };
    const int cbase = e;   // level l + 1 starts where level l ends
    // children that do not all fit the node pool: no node of level l is split (the level's nodes
    // stay leaves, the next level is empty), the status bit reports it, and no slot of the pool
    // is left half-written
    const int total = prefix(nchunks);
    const bool full = cbase + total > node_cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (full) atomicOr(err, (unsigned)ERR_NODE_POOL);
        lvl_start[l + 2] = full ? cbase : cbase + total;
    }
    // a level of few chunks shares each chunk among S blocks: every block of a chunk forms the
    // chunk's offsets (a block scan) and writes the children of its own 1/S of the nodes, so that
    // the child records of the upper levels are written by the whole grid
    const int S = nchunks > 0 ? min(LEVEL_CHUNK, max(1, (int)gridDim.x / nchunks)) : 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int job = blockIdx.x; job < nchunks * S; job += gridDim.x) {
        const int chunk = job / S, part = job - chunk * S;
        const int lo_t = part * LEVEL_CHUNK / S, hi_t = (part + 1) * LEVEL_CHUNK / S;
        const bool mine = (int)threadIdx.x >= lo_t && (int)threadIdx.x < hi_t;
        const int chunk_off = prefix(chunk);
        const int node = s + chunk * LEVEL_CHUNK + threadIdx.x;
        const int nc = node < e ? __ldcg(tmp_cur + (node - s)) : 0;
        // child offsets within the chunk: warp scans, then a scan of the 32 warp totals
        int incl = nc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) sc[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int w = sc[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL, w, o);
                if (lane >= o) w += y;
            }
            sc[lane] = w;
        }
        __syncthreads();
        incl += warp > 0 ? sc[warp - 1] : 0;
        const int off = incl - nc + chunk_off;
        if (COUNT) {
            // the children of this block's nodes occupy [cbase + sc[32], cbase + sc[33])
            if ((int)threadIdx.x == lo_t) sc[32] = off;
            if ((int)threadIdx.x == hi_t - 1) sc[33] = incl + chunk_off;
        }
        __syncthreads();
        if (mine && node < e && nc > 0) {
            const int b = __ldcg(na.begin + node), cnt = __ldcg(na.count + node);
            int bnd[NC + 1];
            bnd[0] = b;
            bnd[NC] = b + cnt;
#pragma unroll
            for (int c = 1; c < NC; ++c) bnd[c] = __ldcg(na.bnd + (size_t)node * (NC - 1) + (c - 1));
            const int fc = cbase + off;
            if (full) {
                na.first[node] = -1;
                na.nchild[node] = 0;
            } else {
                na.first[node] = fc;
                na.nchild[node] = nc;
                const double edge = __ldcg(na.edge + node);
                double cen[D];
#pragma unroll
                for (int k = 0; k < D; ++k) cen[k] = __ldcg(na.center[k] + node);
                int ci = fc;
                for (int c = 0; c < NC; ++c) {
                    if (bnd[c + 1] <= bnd[c]) continue;
                    na.begin[ci] = bnd[c];
                    na.count[ci] = bnd[c + 1] - bnd[c];
                    na.level[ci] = l + 1;
                    na.parent[ci] = node;
                    na.first[ci] = -1;
                    na.nchild[ci] = 0;
                    na.arrive[ci] = 0;
                    na.edge[ci] = edge * 0.5;
#pragma unroll
                    for (int k = 0; k < D; ++k)
                        na.center[k][ci] = __dadd_rn(cen[k], ((c >> k) & 1 ? edge : -edge) * 0.25);
                    ++ci;
                }
            }
        }
        if (COUNT && !full) {
            __syncthreads();   // this block's child records, visible to all its threads
            count_nodes_block<D>(na, nx.keys, nx.n, cbase + sc[32], cbase + sc[33], cbase, l + 1, nx.levels,
                                 nx.lv, nx.leaf_num, nx.lvl_tmp, nx.chunk_sum, nx.trunc);
        }
    }
}

template <int D>
__global__ void __launch_bounds__(LEVEL_CHUNK) level_build_kernel(NodeArrays na, int* lvl_start, int l,
                                                                  const int* tmp_cur, const int* cs_cur,
                                                                  int* cs_clear, int cs_cap, int node_cap,
                                                                  unsigned* err, const int* cs_off)
{
    __shared__ int sc[34];
    __shared__ int red[32];
    build_level<D, false>(na, lvl_start, l, tmp_cur, cs_cur, cs_clear, cs_cap, node_cap, err, sc, red, NextCount{},
                          cs_off);
}

// Exclusive scan of the chunk totals of level l (one block, tiles of 4096 with a carry), with the
// level's total after the last chunk: the chunk offsets level_build_kernel reads.
__global__ void __launch_bounds__(1024) chunk_offsets_kernel(const int* lvl_start, int l, const int* cs, int* off)
{
    __shared__ int wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int nch = (lvl_start[l + 1] - lvl_start[l] + LEVEL_CHUNK - 1) / LEVEL_CHUNK;
    int carry = 0;
    for (int b0 = 0; b0 < nch; b0 += 4096) {
        const int base = b0 + 4 * t;
        int x[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = base + k < nch ? __ldcg(cs + base + k) : 0;
        const int own = x[0] + x[1] + x[2] + x[3];
        int incl = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        __syncthreads();   // the previous tile's readers of wsum are done
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        if (w == 0) {
            int v = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL, v, o);
                if (lane >= o) v += y;
            }
            wsum[lane] = v;
        }
        __syncthreads();
        int run = carry + incl - own + (w > 0 ? wsum[w - 1] : 0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (base + k < nch) off[base + k] = run;
            run += x[k];
        }
        carry += wsum[31];
    }
    if (t == 0) off[nch] = carry;
}

// Bounded grid-wide barrier of a cooperative launch (all blocks resident): the last block to
// arrive resets the count and advances the generation; the others wait for the generation with a
// bounded number of polls.  false when the wait ran out (ERR_TIMEOUT raised); the caller then stops.
constexpr unsigned GRID_WAIT_POLLS = 1u << 20;   // about half a second of 64 ns sleeps and polls
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned* err)
{
    __shared__ int ok;
    __threadfence();   // this thread's writes of the phase, device-wide, before the arrival
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        ok = 1;
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned it = 0;
            while (*vgen == gen) {
                if (++it > GRID_WAIT_POLLS) { atomicOr(err, (unsigned)ERR_TIMEOUT); ok = 0; break; }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Every level of the build in one cooperative launch: the counts of the roots, then per level the
// placement of its children, each block counting the children it placed, with one grid-wide
// barrier per level (the same nodes as the per-level launches, without their launch gaps).
template <int D>
__global__ void __launch_bounds__(LEVEL_CHUNK) levels_fused_kernel(NodeArrays na, const unsigned long long* keys,
                                                                   int n, int* lvl_start, int levels, int lv,
                                                                   int leaf_num, int* tmp0, int* tmp1, int* cs0,
                                                                   int* cs1, int* cs2, int cs_cap, int node_cap,
                                                                   int* trunc, unsigned* err, unsigned* bar,
                                                                   int inject_leave)
{
    __shared__ int sc[34];
    __shared__ int red[32];
    int* tmp[2] = {tmp0, tmp1};
    int* cs[3] = {cs0, cs1, cs2};
    count_level<D, LEVEL_CHUNK>(na, keys, n, lvl_start, 1, levels, lv, leaf_num, tmp[1], cs[1], trunc, red);
    // fault injection for the tests of the barrier's bounded wait (knob 33): block 0 leaves
    // without arriving, so that the other blocks' first wait runs out
    if (inject_leave && blockIdx.x == 0) return;
    for (int l = 1; l <= lv; ++l) {
        if (!grid_barrier(bar, err)) return;
        // an empty level l leaves every deeper level empty: their starts are its end
        const int end = __ldcg(lvl_start + l + 1);
        if (l > 1 && end == __ldcg(lvl_start + l)) {
            if (blockIdx.x == 0)
                for (int q = l + 2 + (int)threadIdx.x; q <= lv + 2; q += (int)blockDim.x) lvl_start[q] = end;
            return;
        }
        // the children of level l, and their counts (level l + 1) by the blocks that placed them
        const NextCount nx{keys, n, levels, lv, leaf_num, tmp[(l + 1) & 1], cs[(l + 1) % 3], trunc};
        build_level<D, true>(na, lvl_start, l, tmp[l & 1], cs[l % 3], cs[(l + 2) % 3], cs_cap, node_cap, err,
                             sc, red, nx);
    }
}

// ---- bottom-up reductions, one tree level per launch -------------------------------------------
// Level l occupies the node range [lvl_start[l], lvl_start[l + 1]) of the breadth-first arrays;
// deeper levels are done first, so a node reads its finished children (no atomics, and the sums
// do not depend on scheduling).

// Kernel size (BHTree::set_kernel, src/bhtree.cpp:206-232): leaves take the maximum h of their
// particles, inner nodes the maximum of their children.
__global__ void ksize_level_kernel(const double* sml, const int* lvl_start, int l, const int* begin,
                                   const int* count, const int* first, const int* nchild, double* ksize)
{
    const int s = lvl_start[l], e = lvl_start[l + 1];
    for (int i = s + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
        double h = 0.0;
        const int fc = first[i];
        if (fc < 0) {
            const int b = begin[i], en = b + count[i];
            for (int j = b; j < en; ++j) h = fmax(h, sml[j]);
        } else {
            const int nc = nchild[i];
            for (int c = 0; c < nc; ++c) h = fmax(h, ksize[fc + c]);
        }
        ksize[i] = h;
    }
}

// Mass and sum of m x per node: leaves sum their particles, inner nodes their children.  The roots
// keep zero mass and centre, as in the reference, whose root never receives them.
template <int D>
__global__ void moments_level_kernel(State st, const int* lvl_start, int l, int R, const int* begin,
                                     const int* count, const int* first, const int* nchild,
                                     double* mass, double* mx0, double* mx1, double* mx2)
{
    double* mx[3] = {mx0, mx1, mx2};
    const int s = lvl_start[l], e = lvl_start[l + 1];
    for (int i = max(s, R) + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x) {
        double m = 0.0, sx[D];
#pragma unroll
        for (int k = 0; k < D; ++k) sx[k] = 0.0;
        const int fc = first[i];
        if (fc < 0) {
            const int b = begin[i], en = b + count[i];
            for (int j = b; j < en; ++j) {
                const double mj = st.f[F_MASS][j];
                m += mj;
#pragma unroll
                for (int k = 0; k < D; ++k) sx[k] += st.f[F_POS + k][j] * mj;
            }
        } else {
            const int nc = nchild[i];
            for (int c = 0; c < nc; ++c) {
                m += mass[fc + c];
#pragma unroll
                for (int k = 0; k < D; ++k) sx[k] += mx[k][fc + c];
            }
        }
        mass[i] = m;
#pragma unroll
        for (int k = 0; k < D; ++k) mx[k][i] = sx[k];
    }
}

// The same sums bottom-up in one launch: every leaf sums its particles, then climbs: it counts
// itself in at its parent after a fence that publishes its sums, and the child that arrives last
// finishes the parent from all its children (in child order, as the level launches do) and climbs
// on.  Every node is finished exactly once, after all its children, and no thread waits for
// another; the counters return to zero.  The roots are not summed.
template <int D>
__global__ void moments_up_kernel(State st, const int* node_total_p, int R, const int* begin, const int* count,
                                  const int* first, const int* nchild, const int* parent, int* arrive,
                                  double* mass, double* mx0, double* mx1, double* mx2, const unsigned* err)
{
    double* mx[3] = {mx0, mx1, mx2};
    if (tree_failed(err)) return;
    const int total = *node_total_p;
    for (int i = R + blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (first[i] >= 0) continue;
        double m = 0.0, sx[D];
#pragma unroll
        for (int k = 0; k < D; ++k) sx[k] = 0.0;
        const int b = begin[i], en = b + count[i];
        for (int j = b; j < en; ++j) {
            const double mj = st.f[F_MASS][j];
            m += mj;
#pragma unroll
            for (int k = 0; k < D; ++k) sx[k] += st.f[F_POS + k][j] * mj;
        }
        mass[i] = m;
#pragma unroll
        for (int k = 0; k < D; ++k) mx[k][i] = sx[k];
        int cur = i;
        for (;;) {
            const int p = parent[cur];
            if (p < R) break;
            __threadfence();
            if (atomicAdd(&arrive[p], 1) != nchild[p] - 1) break;
            __threadfence();
            arrive[p] = 0;
            const int fc = first[p], nc = nchild[p];
            double mp = 0.0, sp[D];
#pragma unroll
            for (int k = 0; k < D; ++k) sp[k] = 0.0;
            for (int c = 0; c < nc; ++c) {
                mp += __ldcg(mass + fc + c);
#pragma unroll
                for (int k = 0; k < D; ++k) sp[k] += __ldcg(mx[k] + fc + c);
            }
            mass[p] = mp;
#pragma unroll
            for (int k = 0; k < D; ++k) mx[k][p] = sp[k];
            cur = p;
        }
    }
}

// centre of mass = (sum m x) / m for every non-root node (src/bhtree.cpp:152).
template <int D>
__global__ void com_finalize_kernel(const int* node_total_p, int R, const double* mass,
                                    double* mx0, double* mx1, double* mx2)
{
    double* mx[3] = {mx0, mx1, mx2};
    const int total = *node_total_p;
    for (int i = R + blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const double m = mass[i];
#pragma unroll
        for (int k = 0; k < D; ++k) mx[k][i] = mx[k][i] / m;
    }
}

// Per-node maximum smoothing length (BHNode::set_kernel, src/bhtree.cpp:206-232), bottom-up in
// one launch by the climb of moments_up_kernel (the maximum does not depend on the order).
__global__ void ksize_up_kernel(const double* sml, const int* node_total_p, const int* begin, const int* count,
                                const int* first, const int* nchild, const int* parent, int* arrive, double* ksize,
                                const unsigned* err)
{
    if (tree_failed(err)) return;
    const int total = *node_total_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (first[i] >= 0) continue;
        double h = 0.0;
        const int b = begin[i], en = b + count[i];
        for (int j = b; j < en; ++j) h = fmax(h, sml[j]);
        ksize[i] = h;
        int cur = i;
        for (;;) {
            const int p = parent[cur];
            if (p < 0) break;
            __threadfence();
            if (atomicAdd(&arrive[p], 1) != nchild[p] - 1) break;
            __threadfence();
            arrive[p] = 0;
            const int fc = first[p], nc = nchild[p];
            double hp = 0.0;
            for (int c = 0; c < nc; ++c) hp = fmax(hp, __ldcg(ksize + fc + c));
            ksize[p] = hp;
            cur = p;
        }
    }
}

// ---- target groups ----------------------------------------------------------------------------
// Each fixed chunk of key-consecutive particles is split at the highest key bit in which its
// first and last particle differ when both halves are less than half as wide as the whole (the
// chunk straddles an octree boundary); the parts are then compacted into the group list in chunk
// order.  One warp per chunk: the lanes take the particles in turn and the extents are minima and
// maxima of the ordered-integer images of the coordinates (exact, and off the FP64 pipe).
constexpr int GROUP_PARTS = 2;

template <int D>
__global__ void split_groups_kernel(State st, const unsigned long long* keys, const int* ck_begin,
                                    const int* ck_count, int nchunks, int* part_begin, int* part_count,
                                    int* nparts)
{
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;   // whole warps
    const int b = ck_begin[c], e = b + ck_count[c];
    int s = e;
    const unsigned long long diff = e - b > 1 ? keys[b] ^ keys[e - 1] : 0ull;
    if (diff) {
        const unsigned long long bit = 1ull << (63 - __clzll((long long)diff));
        int lo = b, hi = e - 1;   // first index with the bit set
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (keys[mid] & bit) hi = mid; else lo = mid + 1;
        }
        if (lo > b) {
            const long long top = dbl_to_ord(1.7976931348623157e308), bottom = dbl_to_ord(-1.7976931348623157e308);
            long long mn[2][D], mx[2][D];
#pragma unroll
            for (int k = 0; k < D; ++k) { mn[0][k] = mn[1][k] = top; mx[0][k] = mx[1][k] = bottom; }
            for (int i = b + lane; i < e; i += 32) {
                const int h = i >= lo;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const long long o = dbl_to_ord(st.f[F_POS + k][i]);
                    mn[h][k] = min(mn[h][k], o);
                    mx[h][k] = max(mx[h][k], o);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        mn[h][k] = min(mn[h][k], __shfl_xor_sync(FULL, mn[h][k], o));
                        mx[h][k] = max(mx[h][k], __shfl_xor_sync(FULL, mx[h][k], o));
                    }
                }
            }
            double ext = 0.0, ea = 0.0, eb = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                ea = fmax(ea, ord_to_dbl(mx[0][k]) - ord_to_dbl(mn[0][k]));
                eb = fmax(eb, ord_to_dbl(mx[1][k]) - ord_to_dbl(mn[1][k]));
                ext = fmax(ext, ord_to_dbl(max(mx[0][k], mx[1][k])) - ord_to_dbl(min(mn[0][k], mn[1][k])));
            }
            if (fmax(ea, eb) < 0.5 * ext) s = lo;
        }
    }
    if (lane == 0) {
        part_begin[(size_t)c * GROUP_PARTS] = b;
        part_count[(size_t)c * GROUP_PARTS] = s - b;
        if (s < e) {
            part_begin[(size_t)c * GROUP_PARTS + 1] = s;
            part_count[(size_t)c * GROUP_PARTS + 1] = e - s;
        }
        nparts[c] = s < e ? 2 : 1;
    }
}

// Exclusive scan of the per-chunk part counts in one block; total to *n_groups.
// Exclusive scan of many counts in two launches: tiles of SCAN_TILE counts scanned by one block
// each (coalesced, four per thread), the tile totals kept; then every block adds the sum of the
// totals before its tile, and the last block writes the grand total.  The single-block scan
// below reads thread-contiguous runs (uncoalesced) and took 0.33 ms for 330,000 counts.
constexpr int SCAN_TILE = 4096;
__global__ void __launch_bounds__(1024) scan_tiles_kernel(int* v, int n, int* tile_sum)
{
    __shared__ int wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int base = blockIdx.x * SCAN_TILE + 4 * t;
    int x[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) x[k] = base + k < n ? v[base + k] : 0;
    const int own = x[0] + x[1] + x[2] + x[3];
    int incl = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        int s = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += y;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    int run = incl - own + (w > 0 ? wsum[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) v[base + k] = run;
        run += x[k];
    }
    if (t == 1023) tile_sum[blockIdx.x] = wsum[31];
}

__global__ void __launch_bounds__(1024) scan_add_kernel(int* v, int n, const int* tile_sum, int ntiles, int* total)
{
    __shared__ int red[32];
    const int t = threadIdx.x;
    int s = 0;
    for (int q = t; q < (int)blockIdx.x; q += blockDim.x) s += tile_sum[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if ((t & 31) == 0) red[t >> 5] = s;
    __syncthreads();
    int off = 0;
    for (int q = 0; q < 32; ++q) off += red[q];
    const int base = blockIdx.x * SCAN_TILE + 4 * t;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k < n) v[base + k] += off;
    if (blockIdx.x == ntiles - 1 && t == 0) *total = off + tile_sum[ntiles - 1];
}

__global__ void scan_parts_kernel(int* nparts, int nchunks, int* n_groups)
{
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (nchunks + 1023) / 1024;
    const int b = t * per, e = min(nchunks, b + per);
    int sum = 0;
    for (int i = b; i < e; ++i) sum += nparts[i];
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = t > 0 ? part[t - 1] : 0;
    for (int i = b; i < e; ++i) {
        const int v = nparts[i];
        nparts[i] = run;
        run += v;
    }
    if (t == 1023) *n_groups = part[1023];
}

__global__ void compact_groups_kernel(const int* part_begin, const int* part_count, const int* offs,
                                      const int* n_groups, int nchunks, int* g_begin, int* g_count)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const int o = offs[c];
    const int cnt = (c + 1 < nchunks ? offs[c + 1] : *n_groups) - o;
    for (int q = 0; q < cnt; ++q) {
        g_begin[o + q] = part_begin[(size_t)c * GROUP_PARTS + q];
        g_count[o + q] = part_count[(size_t)c * GROUP_PARTS + q];
    }
}

// ---- target groups by key-block bisection -------------------------------------------------------
// The groups are the largest aligned key blocks (a key prefix: an octree cell, or the half, quarter
// ... of one, taking one key bit at a time) that hold at most G particles of one run; a block of
// more than G equal keys is cut every G particles.  Unlike fixed chunks of the key order, which
// start anywhere and straddle cells, such a block is compact in space, so its source tile and the
// sources each target tests stay close to the minimum for its size.  Particle i (key order) starts
// a group when it starts a run or when the block of the common key prefix of i - 1 and i holds
// more than G particles (then i - 1 and i fall in different halves of a block that is split).
constexpr int GF_THREADS = 256;

__device__ __forceinline__ bool group_start(const unsigned long long* keys, const int* run, int n, int G, int i)
{
    if (i == 0 || run[i] != run[i - 1]) return true;
    const unsigned long long ki = keys[i];
    const unsigned long long x = keys[i - 1] ^ ki;
    const int L = __clzll((long long)x);   // common leading bits (64: equal keys)
    const unsigned long long mask = L >= 64 ? ~0ull : (L == 0 ? 0ull : (~0ull << (64 - L)));
    // the block [s, e) of the common prefix holds i - 1 and i; it holds more than G particles when
    // i - 1 - G shares the prefix, or else when s + G does
    const int lo = i - 1 - G;
    if (lo >= 0 && ((keys[lo] ^ ki) & mask) == 0ull) {
        if (x != 0ull) return true;
        int a = 0, b = lo;   // a run of more than G equal keys: its first index
        while (a < b) {
            const int m = (a + b) >> 1;
            if (keys[m] == ki) b = m; else a = m + 1;
        }
        return (i - a) % G == 0;
    }
    int a = lo + 1 > 0 ? lo + 1 : 0, b = i - 1;
    while (a < b) {
        const int m = (a + b) >> 1;
        if (((keys[m] ^ ki) & mask) == 0ull) b = m; else a = m + 1;
    }
    if (!(a + G < n && ((keys[a + G] ^ ki) & mask) == 0ull)) return false;
    return x != 0ull || (i - a) % G == 0;
}

// One flag per particle and the flag count of each block of GF_THREADS particles.
__global__ void group_flags_kernel(const unsigned long long* keys, const int* run, int n, int G,
                                   unsigned char* flag, int* blk_count)
{
    __shared__ int wc[GF_THREADS / 32];
    const int i = blockIdx.x * GF_THREADS + threadIdx.x;
    const bool f = i < n && group_start(keys, run, n, G, i);
    if (i < n) flag[i] = f ? 1 : 0;
    const unsigned bal = __ballot_sync(FULL, f);
    if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < GF_THREADS / 32; ++w) s += wc[w];
        blk_count[blockIdx.x] = s;
    }
}

// Group list from the flags: each flagged particle writes its group at the block's offset (the
// exclusive scan of the block counts) plus its rank in the block; the group ends at the next flag
// (at most G particles on).
__global__ void group_write_kernel(const unsigned char* flag, const int* blk_off, int n, int G,
                                   int* g_begin, int* g_count)
{
    constexpr int NW = GF_THREADS / 32;
    __shared__ int wc[NW];
    __shared__ int wfirst[NW + 1];   // first group start of each warp of the block (n when none)
    const int i = blockIdx.x * GF_THREADS + threadIdx.x;
    const bool f = i < n && flag[i];
    const unsigned bal = __ballot_sync(FULL, f);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        wc[w] = __popc(bal);
        wfirst[w] = bal ? (i + __ffs(bal) - 1) : n;
    }
    __syncthreads();
    if (!f) return;
    int o = blk_off[blockIdx.x] + __popc(bal & lanemask_lt());
    for (int q = 0; q < w; ++q) o += wc[q];
    // the group ends at the next start: later in this warp, else in a later warp of the block, else
    // (the block's last group) found by a scan past the block of at most G flags
    const unsigned above = lane < 31 ? bal & (FULL << (lane + 1)) : 0u;
    int e = n;
    if (above) {
        e = i - lane + __ffs(above) - 1;
    } else {
        for (int q = w + 1; q < NW && e == n; ++q) e = wfirst[q];
        if (e == n) {
            e = (blockIdx.x + 1) * GF_THREADS;
            while (e < n && e < i + G && !flag[e]) ++e;
        }
    }
    e = min(e, min(n, i + G));
    g_begin[o] = i;
    g_count[o] = e - i;
}

// ---- FP32 node copies and leaf-relative particle offsets ------------------------------------

struct NodeMirrors {
    float *cf[3], *ef;
    GravNode* grav;
};

template <int D, typename T>
__global__ void node_mirror_kernel(State st, const int* node_total_p, TreeView tv, NodeMirrors nm,
                                   typename Vec4<T>::type* xrel)
{
    const int total = *node_total_p;
    for (int nd = blockIdx.x * blockDim.x + threadIdx.x; nd < total; nd += gridDim.x * blockDim.x) {
        double c[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            c[k] = tv.center[k][nd];
            nm.cf[k][nd] = (float)c[k];
        }
        nm.ef[nd] = __double2float_ru(tv.edge[nd]);
        if (nm.grav) {
            GravNode g;
            float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f}, cc[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const double cm = tv.com[k][nd];
                hi[k] = (float)cm;
                lo[k] = (float)(cm - (double)hi[k]);
                cc[k] = (float)(c[k] - cm);
            }
            g.com = make_float4(hi[0], hi[1], hi[2], (float)(tv.edge[nd] * tv.edge[nd]));
            g.comlo = make_float4(lo[0], lo[1], lo[2], (float)tv.mass[nd]);
            g.link = make_int4(tv.first_child[nd], tv.nchild[nd], tv.begin[nd], tv.count[nd]);
            g.cc = make_float4(cc[0], cc[1], cc[2], 0.f);
            nm.grav[nd] = g;
        }
        if (tv.first_child[nd] >= 0) continue;
        const int b = tv.begin[nd], e = b + tv.count[nd];
        for (int j = b; j < e; ++j) {
            typename Vec4<T>::type q;
            q.x = (T)(st.f[F_POS][j] - c[0]);
            q.y = D > 1 ? (T)(st.f[F_POS + (D > 1 ? 1 : 0)][j] - c[D > 1 ? 1 : 0]) : T(0);
            q.z = D > 2 ? (T)(st.f[F_POS + (D > 2 ? 2 : 0)][j] - c[D > 2 ? 2 : 0]) : T(0);
            q.w = (T)st.f[F_MASS][j];
            xrel[j] = q;
        }
    }
}

// Kernel sizes rounded up to FP32, and the smoothing lengths in T.
template <typename T>
__global__ void kernel_size_mirror_kernel(const int* node_total_p, const double* ksize, float* kf,
                                          const double* sml, int n, T* hm)
{
    const int total = *node_total_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < max(total, n); i += gridDim.x * blockDim.x) {
        if (i < total) kf[i] = __double2float_ru(ksize[i]);
        if (i < n) hm[i] = (T)sml[i];
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------

TreeView tree_view(const Ctx& c)
{
    TreeView t;
    t.begin = c.nd_begin;
    t.count = c.nd_count;
    t.first_child = c.nd_first;
    t.nchild = c.nd_nchild;
    for (int k = 0; k < 3; ++k) {
        t.center[k] = c.nd_center[k]; t.com[k] = c.nd_com[k]; t.cf[k] = c.nd_cf[k];
    }
    t.gn = c.nd_grav;
    t.ef = c.nd_ef;
    t.kf = c.nd_kf;
    t.edge = c.nd_edge;
    t.mass = c.nd_mass;
    t.ksize = c.nd_ksize;
    return t;
}

int tree_alloc(Ctx& c)
{
    const int n = c.n;
    c.node_cap = 5 * n + c.R;   // BHTree::resize: particle_num * 5 (src/bhtree.cpp:42-53)
    const size_t nc = (size_t)c.node_cap;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 8); };
    A((void**)&c.keys, sizeof(unsigned long long) * n);
    A((void**)&c.keys_alt, sizeof(unsigned long long) * n);
    A((void**)&c.perm, sizeof(int) * n);
    A((void**)&c.perm_alt, sizeof(int) * n);
    c.radix_blocks = ceil_div(n, RADIX_TILE);
    A((void**)&c.radix_hist, sizeof(int) * 256 * c.radix_blocks);
    A((void**)&c.radix_dtot, sizeof(int) * 256);
    // key tables (R runs x dim axes x 2^(T+1) entries) of the most levels that fit (none below 4)
    c.key_table_levels = 0;
    for (int t = KEY_TABLE_LEVELS; t >= 4; --t)
        if ((size_t)c.R * c.dim * ((size_t)2 << t) * sizeof(long long) <= KEY_TABLE_BYTES) { c.key_table_levels = t; break; }
    if (c.key_table_levels > 0)
        A((void**)&c.key_table, sizeof(long long) * (size_t)c.R * c.dim * ((size_t)2 << c.key_table_levels));
    A((void**)&c.nd_begin, sizeof(int) * nc);
    A((void**)&c.nd_count, sizeof(int) * nc);
    A((void**)&c.nd_first, sizeof(int) * nc);
    A((void**)&c.nd_nchild, sizeof(int) * nc);
    A((void**)&c.nd_parent, sizeof(int) * nc);
    A((void**)&c.nd_level, sizeof(int) * nc);
    A((void**)&c.nd_arrive, sizeof(int) * nc);
    for (int k = 0; k < c.dim; ++k) {
        A((void**)&c.nd_center[k], sizeof(double) * nc);
        A((void**)&c.nd_com[k], sizeof(double) * nc);
        A((void**)&c.nd_cf[k], sizeof(float) * nc);
    }
    if (c.p.use_gravity) A((void**)&c.nd_grav, sizeof(GravNode) * nc);
    A((void**)&c.nd_ef, sizeof(float) * nc);
    A((void**)&c.nd_kf, sizeof(float) * nc);
    A((void**)&c.nd_edge, sizeof(double) * nc);
    A((void**)&c.nd_mass, sizeof(double) * nc);
    A((void**)&c.nd_ksize, sizeof(double) * nc);
    A((void**)&c.lvl_start, sizeof(int) * (MAX_LEVELS + 2));
    A((void**)&c.lvl_tmp, sizeof(int) * 2 * (size_t)nc);
    A((void**)&c.nd_bnd, sizeof(int) * ((1 << c.dim) - 1) * nc);
    A((void**)&c.chunk_sum, sizeof(int) * 3 * (size_t)(ceil_div(nc, LEVEL_CHUNK) + 1));
    A((void**)&c.chunk_off, sizeof(int) * (size_t)(ceil_div(nc, LEVEL_CHUNK) + 2));
    A((void**)&c.bbox, sizeof(long long) * 2 * 3 * c.R);
    A((void**)&c.node_total, sizeof(int));
    const int max_chunks = n / 32 + c.R + 1;
    // key-block groups: at most one per particle; chunk splits: GROUP_PARTS per chunk
    c.max_groups = n + c.R + 1;
    A((void**)&c.g_begin, sizeof(int) * c.max_groups);
    A((void**)&c.g_count, sizeof(int) * c.max_groups);
    A((void**)&c.ck_begin, sizeof(int) * max_chunks);
    A((void**)&c.ck_count, sizeof(int) * max_chunks);
    A((void**)&c.part_begin, sizeof(int) * GROUP_PARTS * (size_t)max_chunks);
    A((void**)&c.part_count, sizeof(int) * GROUP_PARTS * (size_t)max_chunks);
    A((void**)&c.part_n, sizeof(int) * max_chunks);   // also the block counts of the key-block flags
    A((void**)&c.scan_tiles, sizeof(int) * (max_chunks / SCAN_TILE + 2));
    A((void**)&c.g_flag, sizeof(unsigned char) * ((size_t)n + 1));
    // group plans of the first pair pass: plans for the first plan_cap groups, their leaves in a
    // pool (groups beyond either walk in the pair kernel)
    c.plan_cap = std::min(c.max_groups, n / 8 + c.R + 64);
    c.pool_cap = (int)std::min<long long>(1LL << 30, (c.dim == 1 ? n / 4 : c.dim == 2 ? 2LL * n : 6LL * n) + 4096);
    A((void**)&c.plan, sizeof(GroupPlan) * (size_t)c.plan_cap);
    A((void**)&c.pool_leaves, sizeof(int2) * (size_t)c.pool_cap);
    A((void**)&c.pool_loff, (c.precision == SPHGPU_FP32_PAIR ? 16 : 32) * (size_t)c.pool_cap);
    A((void**)&c.n_groups, sizeof(int));
    if (e != cudaSuccess) {
        c.last_error = std::string("tree allocation: ") + cudaGetErrorString(e);
        return SPHGPU_ERR_CUDA;
    }
    cudaMemset(c.lvl_start, 0, sizeof(int) * (MAX_LEVELS + 2));
    return SPHGPU_OK;
}

void tree_free(Ctx& c)
{
    void* ptrs[] = {c.keys, c.keys_alt, c.perm, c.perm_alt, c.radix_hist, c.key_table, c.chunk_off, c.nd_begin, c.nd_count,
                    c.nd_first, c.nd_nchild, c.nd_parent, c.nd_level, c.nd_arrive, c.nd_center[0],
                    c.nd_center[1], c.nd_center[2], c.nd_com[0], c.nd_com[1], c.nd_com[2],
                    c.nd_edge, c.nd_mass, c.nd_ksize, c.lvl_start, c.lvl_tmp, c.chunk_sum, c.bbox,
                    c.node_total, c.g_begin, c.g_count, c.n_groups, c.nd_cf[0], c.nd_cf[1],
                    c.nd_cf[2], c.nd_ef, c.nd_kf, c.ck_begin, c.ck_count, c.radix_dtot, c.nd_grav, c.nd_bnd, c.part_begin,
                    c.part_count, c.part_n, c.scan_tiles, c.g_flag, c.plan, c.pool_leaves, c.pool_loff};
    for (void* p : ptrs)
        if (p) cudaFree(p);
}

// Inside a step, fields that the stages after the rebuild recompute before reading them need
// no move: PRES, SML, ACC, DENE always; GRADH for ssph/disph; PHI with gravity; the gsph
// gradients with the second-order scheme.
static bool moved_in_step(const Ctx& c, int f)
{
    if (!c.st.f[f]) return false;
    bool recomputed = (f >= F_ACC && f < F_ACC + 3) || f == F_PRES || f == F_DENE || f == F_SML;
    if (f == F_GRADH && c.p.sph_type != 2) recomputed = true;
    if (f == F_PHI && c.p.use_gravity) recomputed = true;
    if (f >= F_GRADD && c.p.sph_type == 2 && c.p.gsph_2nd_order) recomputed = true;
    return !recomputed;
}

// The host side of a step's reorder: the moved fields (and the ids) now live in the alternate
// buffers, which become the state's; the parity of the buffer sets flips.  A replayed step graph
// does the same on the host after its launch (the graph of each parity has its pointers baked in).
void step_reorder_swap(Ctx& c)
{
    for (int f = 0; f < F_COUNT; ++f)
        if (moved_in_step(c, f)) std::swap(c.st.f[f], c.alt.f[f]);
    std::swap(c.st.id, c.alt.id);
    c.parity ^= 1;
}

void launch_reorder_fields(Ctx& c, bool all)
{
    FieldMove fm{};
    for (int f = 0; f < F_COUNT; ++f) {
        if (!c.st.f[f]) continue;
        if (!all && !moved_in_step(c, f)) continue;
        fm.src[fm.nf] = c.st.f[f];
        fm.dst[fm.nf] = c.alt.f[f];
        ++fm.nf;
    }
    fm.isrc[0] = c.st.id; fm.idst[0] = c.alt.id;
    fm.ni = 1;
    if (all) { fm.isrc[1] = c.st.neighbor; fm.idst[1] = c.alt.neighbor; fm.ni = 2; }
    reorder_kernel<<<ceil_div(c.n, 256), 256, 0, c.stream>>>(fm, c.perm, c.n);
    if (!all) {
        // a step's reorder: the sorted copies become the state (no copy back)
        step_reorder_swap(c);
        return;
    }
    // a full reorder outside the step loop copies back, so the buffer assignment stays one of
    // the two that the step graphs were captured with
    FieldMove back{};
    back.nf = fm.nf;
    back.ni = fm.ni;
    for (int q = 0; q < fm.nf; ++q) { back.src[q] = fm.dst[q]; back.dst[q] = const_cast<double*>(fm.src[q]); }
    for (int q = 0; q < fm.ni; ++q) { back.isrc[q] = fm.idst[q]; back.idst[q] = const_cast<int*>(fm.isrc[q]); }
    copy_fields_kernel<<<ceil_div(c.n, 256), 256, 0, c.stream>>>(back, c.n);
}

template <int D>
static void make_tree_d(Ctx& c, bool reorder_all, bool full_depth)
{
    const int n = c.n, R = c.R;
    cudaStream_t s = c.stream;
    TreeView tv = tree_view(c);
    if (!c.pb.on) {
        bbox_init_kernel<<<ceil_div(R * D, 128), 128, 0, s>>>(c.bbox, R, D);
        bbox_kernel<D><<<std::max(1, ceil_div(n, 256 * BBOX_ROWS)), 256, 0, s>>>(c.st, n, c.bbox);
    }
    roots_kernel<D><<<ceil_div(R, 128), 128, 0, s>>>(
        tv, c.nd_center[0], c.nd_center[1], c.nd_center[2], c.nd_edge, c.nd_begin, c.nd_count,
        c.nd_first, c.nd_nchild, c.nd_level, c.nd_parent, c.nd_arrive, c.nd_mass, c.nd_com[0],
        c.nd_com[1], c.nd_com[2], c.bbox, c.d_run_begin, R, c.pb, c.lvl_start);
    const int levels = c.key_levels;
    const int run_shift = D * levels;
    // levels split in this build: all of them with gravity (its node sets are the reference's),
    // at most depth_cap otherwise
    const int lv = (full_depth || c.p.use_gravity || c.depth_cap <= 0) ? levels : std::min(levels, c.depth_cap);
    c.tree_levels = lv;
    // the first levels of every run's centre recursion as a table (knob 34), when it fits; below
    // 2^18 particles the table's launch costs more than the FP64 additions it saves (Gresho 65k:
    // +0.4 % per step with it; KHI 786k -1.4 %, the 10.6M-particle ensemble -1.6 %)
    const bool table = c.key_table && (c.key_table_on == 2 || (c.key_table_on == 1 && n >= (1 << 18)));
    // the table's entries cost about as many FP64 additions as the particles' levels they replace:
    // keep it below a quarter of the particles (a large batch of small runs takes fewer levels)
    int T = table ? std::min(c.key_table_levels, lv) : 0;
    while (T > 0 && (long long)R * D * (2LL << T) * 4 > n) --T;
    if (T < 4) T = 0;
    if (T > 0) {
        const long long total = (long long)R * D * (2 << T);
        key_table_kernel<<<(int)std::min<long long>(ceil_div((int)std::min<long long>(total, 1LL << 30), 256), 4096), 256, 0, s>>>(
            tv, R, D, T, c.key_table);
    }
    keys_kernel<D><<<ceil_div(n, 256), 256, 0, s>>>(c.st, n, tv, levels, lv, run_shift, c.keys, c.perm,
                                                   c.key_table, T);
    // radix sort on the significant bits: the lv digits computed and the run index
    const int shift0 = D * (levels - lv);
    const int bits = D * lv + c.run_bits;
    const int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int shift = shift0 + 8 * p;
        radix_hist_kernel<<<c.radix_blocks, RADIX_THREADS, 0, s>>>(c.keys, n, shift, c.radix_hist, c.radix_blocks);
        radix_scan_columns_kernel<<<256, 1024, 0, s>>>(c.radix_hist, c.radix_blocks, c.radix_dtot);
        radix_scatter_kernel<<<c.radix_blocks, RADIX_THREADS, 0, s>>>(
            c.keys, c.perm, c.keys_alt, c.perm_alt, n, shift, c.radix_hist, c.radix_blocks, c.radix_dtot);
        std::swap(c.keys, c.keys_alt);
        std::swap(c.perm, c.perm_alt);
    }
    launch_reorder_fields(c, reorder_all);
    // nodes, level by level
    NodeArrays na;
    na.begin = c.nd_begin; na.count = c.nd_count; na.first = c.nd_first; na.nchild = c.nd_nchild;
    na.parent = c.nd_parent; na.level = c.nd_level; na.arrive = c.nd_arrive;
    for (int k = 0; k < 3; ++k) na.center[k] = c.nd_center[k];
    na.edge = c.nd_edge;
    na.bnd = c.nd_bnd;
    // nodes the build may use: the pool (5 N + runs), or less under the node-limit knob
    const int pool = c.node_limit > 0 ? std::min(c.node_limit, c.node_cap) : c.node_cap;
    const int grid = std::max(1, std::min(c.num_sms * 4, ceil_div(c.node_cap, LEVEL_CHUNK)));
    const int cgrid = std::max(1, std::min(c.num_sms * 16, ceil_div(c.node_cap, COUNT_THREADS)));
    {
        // child counts of the roots, then one launch per level (children of level l and their counts)
        const int cs_cap = ceil_div(c.node_cap, LEVEL_CHUNK) + 1;
        int* tmp[2] = {c.lvl_tmp, c.lvl_tmp + c.node_cap};
        int* cs[3] = {c.chunk_sum, c.chunk_sum + cs_cap, c.chunk_sum + 2 * cs_cap};
        cudaMemsetAsync(c.chunk_sum, 0, sizeof(int) * 3 * (size_t)cs_cap, s);
        // one cooperative launch for all levels (knob 32), or one launch per level and phase
        int fgrid = 0;
        if (c.fused_levels) {
            int nb = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, levels_fused_kernel<D>, LEVEL_CHUNK, 0) != cudaSuccess) {
                cudaGetLastError();
                nb = 0;
            }
            fgrid = std::min(nb * c.num_sms, std::max(1, ceil_div(c.node_cap, LEVEL_CHUNK)));
        }
        if (fgrid > 0) {
            cudaMemsetAsync(c.d_work + GRID_BAR_SLOT, 0, 2 * sizeof(unsigned), s);
            const unsigned long long* a_keys = c.keys;
            int a_n = n, a_levels = levels, a_lv = lv, a_leaf = c.p.leaf_num, a_cs_cap = cs_cap, a_pool = pool;
            int* a_lvl = c.lvl_start;
            int* a_tr = trunc_flag(c);
            unsigned* a_err = c.d_err;
            unsigned* a_bar = reinterpret_cast<unsigned*>(c.d_work + GRID_BAR_SLOT);
            int a_inject = c.inject_barrier_timeout;
            c.inject_barrier_timeout = 0;   // one build only
            void* args[] = {&na, &a_keys, &a_n, &a_lvl, &a_levels, &a_lv, &a_leaf, &tmp[0], &tmp[1],
                            &cs[0], &cs[1], &cs[2], &a_cs_cap, &a_pool, &a_tr, &a_err, &a_bar, &a_inject};
            cudaLaunchCooperativeKernel((const void*)levels_fused_kernel<D>, dim3(fgrid), dim3(LEVEL_CHUNK), args, 0, s);
        } else {
        level_count_kernel<D><<<cgrid, COUNT_THREADS, 0, s>>>(na, c.keys, n, c.lvl_start, 1, levels, lv,
                                                             c.p.leaf_num, tmp[1], cs[1], trunc_flag(c));
        // chunk offsets from one scan per level: the build's per-chunk block sums are O(chunks)
        // each, which the levels of large 1D batches (thousands of chunks) pay quadratically
        const bool offs = true;
        for (int l = 1; l <= lv; ++l) {
            if (offs) chunk_offsets_kernel<<<1, 1024, 0, s>>>(c.lvl_start, l, cs[l % 3], c.chunk_off);
            level_build_kernel<D><<<grid, LEVEL_CHUNK, 0, s>>>(na, c.lvl_start, l, tmp[l & 1], cs[l % 3],
                                                             cs[(l + 2) % 3], cs_cap, pool, c.d_err,
                                                             offs ? c.chunk_off : nullptr);
            level_count_kernel<D><<<cgrid, COUNT_THREADS, 0, s>>>(na, c.keys, n, c.lvl_start, l + 1, levels, lv,
                                                                 c.p.leaf_num, tmp[(l + 1) & 1], cs[(l + 1) % 3],
                                                                 trunc_flag(c));
        }
        }
    }
    cudaMemcpyAsync(c.node_total, c.lvl_start + lv + 2, sizeof(int), cudaMemcpyDeviceToDevice, s);
    if (c.p.use_gravity) launch_node_moments(c);   // node masses and centres of mass serve gravity only
    if (c.group_rule == 1) {
        // key-block groups of at most group_threads particles
        const int nblk = ceil_div(n, GF_THREADS);
        group_flags_kernel<<<nblk, GF_THREADS, 0, s>>>(c.keys, c.st.run, n, c.group_threads, c.g_flag, c.part_n);
        if (nblk <= 16384) {
            scan_parts_kernel<<<1, 1024, 0, s>>>(c.part_n, nblk, c.n_groups);
        } else {
            const int nt = ceil_div(nblk, SCAN_TILE);
            scan_tiles_kernel<<<nt, 1024, 0, s>>>(c.part_n, nblk, c.scan_tiles);
            scan_add_kernel<<<nt, 1024, 0, s>>>(c.part_n, nblk, c.scan_tiles, nt, c.n_groups);
        }
        group_write_kernel<<<nblk, GF_THREADS, 0, s>>>(c.g_flag, c.part_n, n, c.group_threads, c.g_begin, c.g_count);
    } else {
        // fixed chunks, each split once where it straddles two distant cells
        split_groups_kernel<D><<<ceil_div(c.num_chunks, 8), 256, 0, s>>>(c.st, c.keys, c.ck_begin, c.ck_count,
                                                                       c.num_chunks, c.part_begin, c.part_count,
                                                                       c.part_n);
        if (c.num_chunks <= 16384) {
            scan_parts_kernel<<<1, 1024, 0, s>>>(c.part_n, c.num_chunks, c.n_groups);
        } else {
            const int nt = ceil_div(c.num_chunks, SCAN_TILE);
            scan_tiles_kernel<<<nt, 1024, 0, s>>>(c.part_n, c.num_chunks, c.scan_tiles);
            scan_add_kernel<<<nt, 1024, 0, s>>>(c.part_n, c.num_chunks, c.scan_tiles, nt, c.n_groups);
        }
        compact_groups_kernel<<<ceil_div(c.num_chunks, 128), 128, 0, s>>>(c.part_begin, c.part_count, c.part_n,
                                                                         c.n_groups, c.num_chunks, c.g_begin,
                                                                         c.g_count);
    }
    tv = tree_view(c);
    NodeMirrors nm{};
    for (int k = 0; k < 3; ++k) {
        nm.cf[k] = c.nd_cf[k];
    }
    nm.ef = c.nd_ef;
    nm.grav = c.nd_grav;
    if (c.precision == SPHGPU_FP32_PAIR)
        node_mirror_kernel<D, float><<<c.num_sms * 8, 128, 0, s>>>(c.st, c.node_total, tv, nm, (float4*)c.mir[6]);
    else
        node_mirror_kernel<D, double><<<c.num_sms * 8, 128, 0, s>>>(c.st, c.node_total, tv, nm, (double4_32a*)c.mir[6]);
    c.tree_valid = true;
    c.kernel_size_valid = false;
}

void launch_make_tree(Ctx& c, bool reorder_all, bool full_depth)
{
    if (c.dim == 1) make_tree_d<1>(c, reorder_all, full_depth);
    else if (c.dim == 2) make_tree_d<2>(c, reorder_all, full_depth);
    else make_tree_d<3>(c, reorder_all, full_depth);
}

int tree_depth(Ctx& c)
{
    int ls[MAX_LEVELS + 2];
    const int nl = c.tree_levels + 3;
    cudaMemcpyAsync(ls, c.lvl_start, sizeof(int) * nl, cudaMemcpyDeviceToHost, c.stream);
    cudaStreamSynchronize(c.stream);
    int depth = 1;
    for (int l = 1; l + 1 < nl; ++l)
        if (ls[l + 1] > ls[l]) depth = l;
    return depth;
}

void launch_node_moments(Ctx& c)
{
    const int grid = c.num_sms * 8;
    if (c.dim == 1)
        moments_up_kernel<1><<<grid, 256, 0, c.stream>>>(c.st, c.node_total, c.R, c.nd_begin, c.nd_count, c.nd_first, c.nd_nchild, c.nd_parent, c.nd_arrive, c.nd_mass, c.nd_com[0], c.nd_com[1], c.nd_com[2], c.d_err);
    else if (c.dim == 2)
        moments_up_kernel<2><<<grid, 256, 0, c.stream>>>(c.st, c.node_total, c.R, c.nd_begin, c.nd_count, c.nd_first, c.nd_nchild, c.nd_parent, c.nd_arrive, c.nd_mass, c.nd_com[0], c.nd_com[1], c.nd_com[2], c.d_err);
    else
        moments_up_kernel<3><<<grid, 256, 0, c.stream>>>(c.st, c.node_total, c.R, c.nd_begin, c.nd_count, c.nd_first, c.nd_nchild, c.nd_parent, c.nd_arrive, c.nd_mass, c.nd_com[0], c.nd_com[1], c.nd_com[2], c.d_err);
    if (c.dim == 1) com_finalize_kernel<1><<<grid, 256, 0, c.stream>>>(c.node_total, c.R, c.nd_mass, c.nd_com[0], c.nd_com[1], c.nd_com[2]);
    else if (c.dim == 2) com_finalize_kernel<2><<<grid, 256, 0, c.stream>>>(c.node_total, c.R, c.nd_mass, c.nd_com[0], c.nd_com[1], c.nd_com[2]);
    else com_finalize_kernel<3><<<grid, 256, 0, c.stream>>>(c.node_total, c.R, c.nd_mass, c.nd_com[0], c.nd_com[1], c.nd_com[2]);
}

void launch_set_kernel_size(Ctx& c)
{
    if (c.dim >= 2) {
        ksize_up_kernel<<<c.num_sms * 8, 256, 0, c.stream>>>(c.st.f[F_SML], c.node_total, c.nd_begin, c.nd_count,
                                                            c.nd_first, c.nd_nchild, c.nd_parent, c.nd_arrive, c.nd_ksize,
                                                            c.d_err);
    } else {
        // 1D trees are binary and deep, with leaves of a few particles: the climb's fence and atomic per
        // node cost more there than one launch per level
        for (int l = c.tree_levels + 1; l >= 1; --l)
            ksize_level_kernel<<<c.num_sms * 8, 256, 0, c.stream>>>(c.st.f[F_SML], c.lvl_start, l, c.nd_begin,
                                                                   c.nd_count, c.nd_first, c.nd_nchild,
                                                                   c.nd_ksize);
    }
    if (c.precision == SPHGPU_FP32_PAIR)
        kernel_size_mirror_kernel<float><<<c.num_sms * 8, 256, 0, c.stream>>>(c.node_total, c.nd_ksize, c.nd_kf, c.st.f[F_SML], c.n, (float*)c.mir[7]);
    else
        kernel_size_mirror_kernel<double><<<c.num_sms * 8, 256, 0, c.stream>>>(c.node_total, c.nd_ksize, c.nd_kf, c.st.f[F_SML], c.n, (double*)c.mir[7]);
    c.kernel_size_valid = true;
}

int build_groups(Ctx& c)
{
    const int G = 32 * c.gw_pre;
    std::vector<int> cb, cc;
    for (int r = 0; r < c.R; ++r)
        for (int b = c.run_begin[r]; b < c.run_begin[r + 1]; b += G) {
            cb.push_back(b);
            cc.push_back(std::min(G, c.run_begin[r + 1] - b));
        }
    const int nck = (int)cb.size();
    const int ng = nck;   // until the first tree build splits them, the groups are the chunks
    if (ng > c.max_groups) return SPHGPU_ERR_CAPACITY;
    // stream-ordered copies: later kernels on the library's (non-blocking) stream read these
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c.ck_begin, cb.data(), sizeof(int) * nck, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c.ck_count, cc.data(), sizeof(int) * nck, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c.g_begin, cb.data(), sizeof(int) * nck, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c.g_count, cc.data(), sizeof(int) * nck, cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c.n_groups, &ng, sizeof(int), cudaMemcpyHostToDevice, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);   // the host vectors go out of scope
    if (e != cudaSuccess) {
        c.last_error = std::string("group list: ") + cudaGetErrorString(e);
        return SPHGPU_ERR_CUDA;
    }
    c.group_threads = G;
    c.num_chunks = nck;
    c.num_groups = ng;
    c.tree_valid = false;
    return SPHGPU_OK;
}

}  // namespace sphgpu
