// Neighbour-set export for parity checks: for the current smoothing lengths, the sets
// {j : r_ij^2 < h_i^2} (is_ij = 0) and {j : r_ij^2 < max(h_i^2, h_j^2)} (is_ij = 1) of
// exhaustive_search (src/exhaustive_search.cpp:11-42), decided with the reference's FP64
// arithmetic, gathered through the octree walk of group.cuh, written in the caller's order.
#include "context.cuh"

namespace sphgpu {

namespace {

template <typename T>
struct NbArgs {
    State st;
    const typename Vec4<T>::type* xrel;
    const T* hmir;
    TreeView tv;
    Periodic pb;
    SmemLayout L;
    GroupWork work;
    int is_ij;
    int* counts;   // caller order
    int* list;     // caller order, cap per particle
    int cap;
};

template <int D, typename T>
__global__ void __launch_bounds__(256) neighbors_kernel(NbArgs<T> a)
{
    if (tree_failed(a.work.err)) return;   // the octree of this step was not completed
    extern __shared__ __align__(16) unsigned char smem[];
    const SmemLayout L = a.L;
    GroupMisc* gm = reinterpret_cast<GroupMisc*>(smem + L.off_misc);
    const Tile<T> tile = tile_of<T>(smem, L);
    const State& st = a.st;
    const int t = threadIdx.x;
    for (;;) {
        int gb, gn;
        if (!next_group(gm, a.work, gb, gn)) break;
        if (gn == 0) continue;   // the unused half of an unsplit chunk
        const bool active = t < gn;
        const int i = gb + (active ? t : 0);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = st.f[F_POS + k][i];
        const double hi = st.f[F_SML][i];
        group_box<D>(gm, xi, active, hi, a.pb);
        const int run = st.run[gb];
        if (!group_walk<D, T>(smem, L, gm, a.tv, run, a.is_ij != 0, a.pb)) { report_overflow(a.work, gb, gn, gm); continue; }
        {
            BoxAccept<D, T> box;
            box.init(gm);
            const T Rt = to_T_up<T>(gm->R);
            const int is_ij = a.is_ij;
            const T* hmir = a.hmir;
            const int ntile = stage_sources<D, T>(smem, L, gm, a.xrel, tile, [&](int j, const T* off) {
                T r = Rt;
                if (is_ij) { const T hj = hmir[j]; r = r > hj ? r : hj; }
                return box(off, r);
            }, [&](int) { return T(0); });
            if (ntile < 0) { report_overflow(a.work, gb, gn, gm); continue; }
            gm->ntile = ntile;
        }
        const int ntile = gm->ntile;
        if (!active) continue;
        const double hi2 = __dmul_rn(hi, hi);
        const int id_i = st.id[i];
        int cnt = 0;
        for (int s = 0; s < ntile; ++s) {
            const int j = tile.idx[s];
            const double r2 = exact_r2<D>(st, xi, j, a.pb);
            double lim = hi2;
            if (a.is_ij) {
                const double hj = st.f[F_SML][j];
                lim = fmax(hi2, __dmul_rn(hj, hj));
            }
            if (r2 < lim) {
                if (cnt < a.cap) a.list[(size_t)id_i * a.cap + cnt] = st.id[j];
                ++cnt;
            }
        }
        a.counts[id_i] = cnt;
        if (a.list && cnt > a.cap) atomicOr(a.work.err, (unsigned)ERR_LIST);
    }
}

template <int D, typename T>
void run_neighbors(Ctx& c, int is_ij, int* d_counts, int* d_list, int cap)
{
    using V4 = typename Vec4<T>::type;
    reset_work_counters(c);
    NbArgs<T> a{};
    a.st = c.st;
    a.xrel = (const V4*)c.mir[6];
    a.hmir = (const T*)c.mir[7];
    a.tv = tree_view(c);
    a.pb = c.pb;
    a.is_ij = is_ij;
    a.counts = d_counts;
    a.list = d_list;
    a.cap = cap;
    auto kern = neighbors_kernel<D, T>;
    launch_pair_passes<NbArgs<T>>(c, (const void*)kern, a, D == 1 ? 128 : 1024, sizeof(V4), sizeof(T),
        [](const void* k, int grid, int block, size_t smem, cudaStream_t st, NbArgs<T>& args) {
            reinterpret_cast<void (*)(NbArgs<T>)>(const_cast<void*>(k))<<<grid, block, smem, st>>>(args);
        });
}

}  // namespace

void launch_neighbors(Ctx& c, int is_ij, int* d_counts, int* d_list, int cap)
{
    const bool f32 = c.precision == SPHGPU_FP32_PAIR;
    if (c.dim == 1) { if (f32) run_neighbors<1, float>(c, is_ij, d_counts, d_list, cap); else run_neighbors<1, double>(c, is_ij, d_counts, d_list, cap); }
    else if (c.dim == 2) { if (f32) run_neighbors<2, float>(c, is_ij, d_counts, d_list, cap); else run_neighbors<2, double>(c, is_ij, d_counts, d_list, cap); }
    else { if (f32) run_neighbors<3, float>(c, is_ij, d_counts, d_list, cap); else run_neighbors<3, double>(c, is_ij, d_counts, d_list, cap); }
}

}  // namespace sphgpu
