// Host-side context of one sphgpu simulation (or batch of runs) and the launchers each
// translation unit provides.
#pragma once

#include <algorithm>
#include <string>
#include <vector>

#include "common.cuh"
#include "group.cuh"

namespace sphgpu {

struct Ctx {
    // configuration
    sphgpu_params p{};
    int dim = 0;
    int n = 0;
    int R = 1;                      // number of runs
    int precision = SPHGPU_FP32_PAIR;
    int key_levels = 0;             // digits per key = maxTreeLevel
    int run_bits = 0;
    Periodic pb{};
    cudaStream_t stream = nullptr;
    int device = 0;
    int num_sms = 0;

    // particle state (key order) and its double buffer
    State st{}, alt{};
    std::vector<int> run_begin;     // host copy, R+1 entries
    int* d_run_begin = nullptr;

    // sort
    unsigned long long *keys = nullptr, *keys_alt = nullptr;
    int *perm = nullptr, *perm_alt = nullptr;
    int* radix_hist = nullptr;      // 256 * max blocks
    int radix_blocks = 0;

    // tree (breadth-first node arrays)
    int node_cap = 0;
    int *nd_begin = nullptr, *nd_count = nullptr, *nd_first = nullptr, *nd_nchild = nullptr;
    int *nd_parent = nullptr, *nd_level = nullptr, *nd_arrive = nullptr;
    double *nd_center[3] = {nullptr, nullptr, nullptr}, *nd_edge = nullptr, *nd_mass = nullptr;
    double *nd_com[3] = {nullptr, nullptr, nullptr}, *nd_ksize = nullptr;
    int* lvl_start = nullptr;       // device, MAX_LEVELS + 2 entries
    int* lvl_tmp = nullptr;         // per-node child counts of the frontier
    int* chunk_sum = nullptr;       // per-1024-node chunk sums
    long long* bbox = nullptr;      // per run: D mins then D maxs (ordered-int images)
    int* node_total = nullptr;      // device: number of nodes built

    // target groups
    int group_threads = 32;         // group size used to build the current group list
    int* g_begin = nullptr;
    int* g_count = nullptr;
    int* n_groups = nullptr;        // device counter
    int max_groups = 0;

    // per-run scalars on the device
    double* d_time = nullptr;
    double* d_dt = nullptr;
    long long* d_hvs = nullptr;     // h / v_sig minimum (ordered-int image)
    long long* d_dtmin = nullptr;   // force-criterion minimum (ordered-int image)
    double* d_sums = nullptr;       // energy/momentum partial sums
    unsigned* d_err = nullptr;      // status bits
    int* d_newton_fail = nullptr;

    // key-ordered mirrors of source fields in the pair type (sized for FP64)
    void* mir[16] = {nullptr};
    // persistent-kernel work counters and the overflow group list
    int* d_work = nullptr;          // 16 counters
    int* d_ovf_list = nullptr;      // max_groups entries

    // staging buffer for field transfers
    double* d_stage = nullptr;
    size_t stage_bytes = 0;
    unsigned char* d_aos = nullptr;
    size_t aos_bytes = 0;
    unsigned char* d_flush = nullptr;   // L2 flush buffer of the benchmark helper
    size_t flush_bytes = 0;

    // state flags
    bool first_pre = true;
    bool tree_valid = false;
    bool kernel_size_valid = false;

    // schedule knobs
    int gw_pre = 1, gw_fluid = 1, gw_grav = 1;
    int tile_cap = 0;               // 0 = automatic
    int autotune = 1;
    bool tuned = false;

    // CUDA graph of one integrate() step
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    bool use_graph = true;
    bool warm = false;
    int graph_kernels = 0;          // kernel nodes of the captured step

    // stage timing
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool timing = false;
    double stage_ms[5] = {0, 0, 0, 0, 0};

    std::string last_error;
};

// ---- tree.cu
int tree_alloc(Ctx& c);
void tree_free(Ctx& c);
void launch_make_tree(Ctx& c, bool reorder_all);
void launch_set_kernel_size(Ctx& c);
void launch_node_moments(Ctx& c);
TreeView tree_view(const Ctx& c);
void launch_reorder_fields(Ctx& c, bool all);

// ---- pre_dD.cu / fluid_dD.cu / gravity.cu
template <int D>
void launch_pre_dim(Ctx& c, bool initial);
template <int D>
void launch_fluid_dim(Ctx& c);
void launch_pre(Ctx& c, bool initial);
void launch_fluid(Ctx& c);
void launch_gravity(Ctx& c);
void launch_gravity_mirror(Ctx& c);
void launch_neighbors(Ctx& c, int is_ij, int* d_counts, int* d_list, int cap);

// ---- integrate.cu
void launch_timestep(Ctx& c);
void launch_predict(Ctx& c);
void launch_correct(Ctx& c);
void launch_init_fields(Ctx& c);
void launch_update_time(Ctx& c);
void launch_energy(Ctx& c, double* d_out);  // d_out: R * (4 + 3) doubles

// shared launch helpers (api.cu)
inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
int max_optin_smem(const Ctx& c);
int kernel_occupancy(const void* kern, int threads, size_t smem);
void reset_work_counters(Ctx& c);
void set_global_error(const std::string& text);   // text of sphgpu_last_error(NULL)

// The largest source tile that fits the opt-in shared memory next to the walk capacities of the
// overflow pass.
inline int big_tile_cap(const Ctx& c, int gt, int elt4, int stack_cap, int leaf_cap)
{
    const SmemLayout L0 = make_layout(gt, 0, elt4, stack_cap, leaf_cap);
    const size_t per = (size_t)elt4 + sizeof(int) + (size_t)gt / 8;
    size_t cap = ((size_t)max_optin_smem(c) - L0.total - 64) / per;
    cap = cap / 32 * 32;
    if (cap > 16384) cap = 16384;
    return (int)cap;
}

}  // namespace sphgpu
