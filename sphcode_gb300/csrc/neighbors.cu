// Neighbour-set export for parity checks: for the current smoothing lengths, the sets
// {j : r_ij^2 < h_i^2} (is_ij = 0) and {j : r_ij^2 < max(h_i^2, h_j^2)} (is_ij = 1) of
// exhaustive_search (src/exhaustive_search.cpp:11-42), decided with the reference's FP64
// arithmetic, gathered through the octree walk of group.cuh, written in the caller's order.
#include "context.cuh"

namespace sphgpu {

namespace {

struct NbArgs {
    State st;
    TreeView tv;
    Periodic pb;
    SmemLayout L;
    GroupWork work;
    int is_ij;
    int* counts;   // caller order
    int* list;     // caller order, cap per particle
    int cap;
};

template <int D>
__global__ void __launch_bounds__(256) neighbors_kernel(NbArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const SmemLayout L = a.L;
    GroupMisc* gm = reinterpret_cast<GroupMisc*>(smem + L.off_misc);
    const Tile<double> tile = tile_of<double>(smem, L);
    const State& st = a.st;
    const int t = threadIdx.x;
    for (;;) {
        const int g = next_group(gm, a.work);
        if (g < 0) break;
        const int gb = a.work.g_begin[g], gn = a.work.g_count[g];
        const bool active = t < gn;
        const int i = gb + (active ? t : 0);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = st.f[F_POS + k][i];
        const double hi = st.f[F_SML][i];
        group_box<D>(gm, xi, active, hi, a.pb);
        const int run = st.run[gb];
        if (!group_walk<D>(smem, L, gm, a.tv, run, a.is_ij != 0, a.pb)) { report_overflow(a.work, g); continue; }
        {
            const double R = gm->R;
            const int is_ij = a.is_ij;
            double he[D];
#pragma unroll
            for (int k = 0; k < D; ++k) he[k] = gm->he[k];
            const int ntile = stage_sources<D, double>(smem, L, gm, st, a.pb, tile, [&](int j, const double* off) {
                const double r = is_ij ? fmax(R, st.f[F_SML][j]) : R;
#pragma unroll
                for (int k = 0; k < D; ++k)
                    if (fabs(off[k]) > (he[k] + r) * (1.0 + 1e-12)) return false;
                return true;
            }, [&](int) { return 0.0; });
            if (ntile < 0) { report_overflow(a.work, g); continue; }
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

template <int D>
void run_neighbors(Ctx& c, int is_ij, int* d_counts, int* d_list, int cap)
{
    reset_work_counters(c);
    NbArgs a{};
    a.st = c.st;
    a.tv = tree_view(c);
    a.pb = c.pb;
    a.is_ij = is_ij;
    a.counts = d_counts;
    a.list = d_list;
    a.cap = cap;
    const int gt = c.group_threads;
    auto kern = neighbors_kernel<D>;
    cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_optin_smem(c));
    a.L = make_layout(gt, D == 1 ? 128 : 1024, sizeof(double4_32a), 256, 256);
    a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + 0, nullptr, nullptr,
                       c.d_ovf_list, c.d_work + 1, c.d_err};
    kern<<<c.num_sms * 2, gt, a.L.total, c.stream>>>(a);
    const int big = big_tile_cap(c, gt, sizeof(double4_32a), 1024, 2048);
    a.L = make_layout(gt, big, sizeof(double4_32a), 1024, 2048);
    a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + 2, c.d_ovf_list, c.d_work + 1,
                       nullptr, nullptr, c.d_err};
    kern<<<c.num_sms, gt, a.L.total, c.stream>>>(a);
}

}  // namespace

void launch_neighbors(Ctx& c, int is_ij, int* d_counts, int* d_list, int cap)
{
    if (c.dim == 1) run_neighbors<1>(c, is_ij, d_counts, d_list, cap);
    else if (c.dim == 2) run_neighbors<2>(c, is_ij, d_counts, d_list, cap);
    else run_neighbors<3>(c, is_ij, d_counts, d_list, cap);
}

}  // namespace sphgpu
