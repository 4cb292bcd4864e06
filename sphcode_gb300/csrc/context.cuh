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
    int* radix_dtot = nullptr;      // 256 digit totals
    long long* key_table = nullptr; // centres of the first key levels per run and axis (tree.cu)
    int key_table_on = 1;           // knob 34: key table 0 off, 1 from 2^18 particles, 2 always
    int key_table_levels = 0;       // levels the allocated table holds
    int radix_blocks = 0;

    // tree (breadth-first node arrays)
    int node_cap = 0;
    int *nd_begin = nullptr, *nd_count = nullptr, *nd_first = nullptr, *nd_nchild = nullptr;
    int *nd_parent = nullptr, *nd_level = nullptr, *nd_arrive = nullptr;
    double *nd_center[3] = {nullptr, nullptr, nullptr}, *nd_edge = nullptr, *nd_mass = nullptr;
    double *nd_com[3] = {nullptr, nullptr, nullptr}, *nd_ksize = nullptr;
    float *nd_cf[3] = {nullptr, nullptr, nullptr}, *nd_ef = nullptr, *nd_kf = nullptr;
    GravNode* nd_grav = nullptr;    // Barnes-Hut node records (gravity only)
    int* lvl_start = nullptr;       // device, MAX_LEVELS + 2 entries
    int* lvl_tmp = nullptr;         // per-node child counts of the frontier
    int* nd_bnd = nullptr;          // per split node: its inner child boundaries (2^D - 1 ints)
    int* chunk_sum = nullptr;       // per-1024-node chunk sums
    int* chunk_off = nullptr;       // their exclusive scan for one level (per-level launches)
    long long* bbox = nullptr;      // per run: D mins then D maxs (ordered-int images)
    int* node_total = nullptr;      // device: number of nodes built

    // target groups: fixed chunks of group_threads key-consecutive particles of one run
    int group_threads = 32;         // group size of the current group list
    int* g_begin = nullptr;
    int* g_count = nullptr;
    int* n_groups = nullptr;        // device copy of the group count
    int max_groups = 0;
    int num_groups = 0;
    int* ck_begin = nullptr;        // fixed chunks of group_threads particles per run
    int* ck_count = nullptr;
    int num_chunks = 0;
    int *part_begin = nullptr, *part_count = nullptr, *part_n = nullptr;   // split scratch
    int* scan_tiles = nullptr;      // tile totals of the two-launch scan of part_n
    unsigned char* g_flag = nullptr;   // key-block groups: group-start flag per particle
    // group formation (knob 30): 1 the largest aligned key blocks of at most group_threads
    // particles (default in 2D and 3D), 0 fixed chunks of group_threads particles, each split once
    // where it straddles two distant cells (default in 1D, where a chunk is an interval)
    int group_rule = 1;

    // per-run scalars on the device
    double* d_time = nullptr;
    double* d_dt = nullptr;
    long long* d_hvs = nullptr;     // h / v_sig minimum (ordered-int image)
    long long* d_dtmin = nullptr;   // force-criterion minimum (ordered-int image)
    int* d_emin = nullptr;          // FP32 estimate of the force-criterion minimum (float bits)
    double* d_sums = nullptr;       // energy/momentum partial sums
    unsigned* d_err = nullptr;      // status bits
    int* d_newton_fail = nullptr;

    // key-ordered mirrors of source fields in the pair type (sized for FP64):
    // 0 Pre {v, c}, 1 Pre u, 2-4 Fluid records, 5 gsph gradients,
    // 6 {x - leaf centre, m} (tree build), 7 h (end of PreInteraction), 8 the smoothing-length
    // guess of the current PreInteraction (written by its first pass, read by the later ones)
    void* mir[16] = {nullptr};
    // persistent-kernel work counters and the overflow group list
    int* d_work = nullptr;          // 64 ints: pair-kernel pass p uses [2p] work, [2p+1] ranges left;
                                    // [48..52] the last range no pass could fit
    int2* d_ovf_list = nullptr;     // target ranges left by a pass (two lists, used alternately)
    int2* d_ovf_list2 = nullptr;
    int ovf_cap = 0;                // capacity of each list

    // staging buffer for field transfers
    double* d_stage = nullptr;
    size_t stage_bytes = 0;
    unsigned char* d_aos = nullptr;
    size_t aos_bytes = 0;
    size_t aos_stage_stride = 0;    // stride of the records the staging buffer holds (0: none)
    bool aos_reuse = false;         // knob 19: downloads take the members outside the layout from
                                    // the last upload's records instead of reading them again
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
    unsigned tune_rejects = 0;      // status bits of tuning candidates that were rejected

    // CUDA graphs of one integrate() step, one per parity of the field buffers: a step's reorder
    // swaps the moved fields between the state's buffers and the alternate ones (step_reorder_swap),
    // so consecutive steps alternate between two pointer sets
    int parity = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_epoch_of[2] = {-1, -1};   // epoch each parity's graph was captured in
    bool use_graph = true;
    bool warm = false;
    int graph_kernels = 0;          // kernel nodes of the captured step
    int graph_epoch = 0;            // bumped whenever captured graphs go stale
    // graphs of one reversed step per parity, keyed by the adjoint buffers they were captured with
    cudaGraphExec_t adj_graph[2] = {nullptr, nullptr};
    const void* adj_key[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    const void* adj_warm_key[3] = {nullptr, nullptr, nullptr};
    int adj_epoch[2] = {-1, -1};

    // stage timing
    cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool timing = false;
    double stage_ms[5] = {0, 0, 0, 0, 0};
    int stage_ovf[2] = {0, 0};      // groups sent to the overflow pass by Pre / Fluid (timing mode)
    int tile_cap_pre = 0;           // per-stage source tile capacities (0 = automatic)
    int pass2_scale = 2;            // tile of the second pair pass, in multiples of the first
    bool fixed_dt = false;          // steps keep the dt set by the caller (no TimeStep)
    // octree levels split in a step's tree build (0: all key levels).  Without gravity the tree
    // only serves the neighbour walks, whose sets do not depend on where the splitting stops;
    // sphgpu_initialize sets it two levels below the initial tree's depth, and a build that had
    // to stop splitting early raises it (trunc_flag).
    int depth_cap = 0;
    unsigned last_trunc = 0;        // capped-tree flag read by the last finish()
    int tree_levels = 0;            // split levels of the last build
    // capacity limits below the allocated ones (0: none), for callers that bound the work of a
    // stage and for tests of the capacity statuses: the source tile of every pair pass (knob 22)
    // and the octree node pool (knob 23)
    int tile_limit = 0;
    int node_limit = 0;
    // tuner trials (in trial order, bit k = trial k) treated as if they had raised the tile
    // status bit: host-side fault injection for tests of the tuner's rejection path (knob 24)
    unsigned tune_fail_mask = 0;
    // work counters of the pair kernels (knob 25; sphgpu_pair_counters): off in timed runs
    bool count_work = false;
    int leaf_cap1 = 0;              // leaf-list capacity of the first pair pass (knob 27; 0: by dimension)
    int pair_sched = 0;             // pair-kernel schedule (knob 28, see launch_pair_passes)
    int bulk_stage = 0;             // tile staging by bulk asynchronous copies (knob 29)
    // group plans (knob 31, bit 0 FluidForce, bit 1 PreInteraction): the first pair pass takes each
    // group's box and leaves from a walk kernel launched ahead of it (one warp per group), instead
    // of walking with one warp of its CTA.  Off by default: measured equal or slower (the walk of
    // one CTA is hidden behind the pair work of the SM's other CTAs)
    int prewalk = 0;
    // the tree's levels in one cooperative launch with grid-wide barriers (knob 32), instead of two
    // launches per level
    int fused_levels = 1;
    // inside run_step: predict leaves the sound speed to the mirror kernels of Pre and Fluid
    bool sound_from_ene = false;
    // the last PreInteraction wrote FluidForce's source records (cleared by FluidForce)
    bool fluid_records_fresh = false;
    // gravity work items (knob 35): 0 the pair kernels' target groups in 32-target pieces, 1 fixed
    // 32-particle chunks of each run's key order (every lane of a warp holds a target; default,
    // Evrard 2^20 gravity about 10 % faster than over the groups' partly filled pieces)
    int gravity_items = 1;
    int* d_gchunk_begin = nullptr;
    int* d_gchunk_count = nullptr;
    int* d_gchunk_n = nullptr;
    int inject_barrier_timeout = 0; // knob 33: the next fused level build's block 0 leaves early (tests)
    GroupPlan* plan = nullptr;
    int plan_cap = 0;
    int2* pool_leaves = nullptr;
    void* pool_loff = nullptr;      // pool_cap four-vectors of the pair type (sized for FP64)
    int pool_cap = 0;
    unsigned long long* d_counters = nullptr;   // PAIR_COUNTERS entries

    // adjoint scratch (allocated on the first adjoint call)
    double* adj_buf = nullptr;      // ADJ_SLOTS x n doubles
    void* adj_mir = nullptr;        // ADJ_MIRRORS x n four-vectors of the pair type
    double* adj_partials = nullptr; // block partials of the avAlpha adjoint

    std::string last_error;
};

// ---- tree.cu
int tree_alloc(Ctx& c);
void tree_free(Ctx& c);
void launch_make_tree(Ctx& c, bool reorder_all, bool full_depth = false);
int tree_depth(Ctx& c);            // deepest level holding nodes in the last build (synchronises)
void launch_set_kernel_size(Ctx& c);
void launch_node_moments(Ctx& c);
TreeView tree_view(const Ctx& c);
void launch_reorder_fields(Ctx& c, bool all);
void step_reorder_swap(Ctx& c);
inline int* trunc_flag(const Ctx& c) { return reinterpret_cast<int*>(c.d_err + 1); }
inline bool step_graph_ready(const Ctx& c, int p) { return c.graph[p] && c.graph_epoch_of[p] == c.graph_epoch; }
int build_groups(Ctx& c);          // host: fixed chunks per run, uploaded to the device

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

// ---- adjoint_dD.cu
// Scratch slots of n doubles each (key order) of the adjoint passes.
enum AdjSlot : int {
    AS_RHOH = 0, AS_RHOHH = 1, AS_DV = 2, AS_DVH = 3, AS_RT = 4, AS_RTH = 7,
    AL_X = 10, AL_V = 13, AL_RHO = 16, AL_P = 17, AL_G = 18, AL_H = 19, AL_C = 20, AL_B = 21,
    AL_ALPHA = 22, AU_LOC = 23, AG_X = 24, AG_V = 27,
    AS_N = 30, AS_NH = 31, AS_NHH = 32, AS_YH = 33, AS_YHH = 34, AL_U = 35, AG_U = 36,   // pressure-energy form
    ADJ_SLOTS = 37
};
constexpr int ADJ_MIRRORS = 7;       // a0..a3, w0..w2 (one four-vector of the pair type each)
constexpr int ADJ_PARTIALS = 1024;   // block partials of the avAlpha adjoint

template <int D>
void launch_adjoint_dim(Ctx& c, double* adj, const double* dens_bar, double* alpha_bar, bool initial);

// ---- integrate.cu
void launch_timestep(Ctx& c);
void launch_predict(Ctx& c, bool store_sound = true);
void launch_correct(Ctx& c);
void launch_init_fields(Ctx& c);
void launch_update_time(Ctx& c);
void launch_energy(Ctx& c, double* d_out);  // d_out: R * (4 + 3) doubles

// shared launch helpers (api.cu)
inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
int max_optin_smem(const Ctx& c);
int kernel_occupancy(const void* kern, int threads, size_t smem);
void reset_work_counters(Ctx& c);
void check_tree_cap(Ctx& c);
void set_global_error(const std::string& text);   // text of sphgpu_last_error(NULL)

// Passes of a CTA-per-group pair kernel.  Pass 1 runs every group with the tuned capacities at
// full occupancy and lists the target ranges that do not fit.  The next log2(G) + 1 passes run
// them with a larger tile (pass2_scale times the first) and larger walk capacities, passing a
// range that still does not fit on as its two halves, so that ranges come down to single targets
// (whose search box is just their own search sphere).  The last two passes run what is left with
// the largest tile the shared memory holds, one CTA per SM.  (Splitting a failing range into
// pieces of 32 targets and then into single targets, with fewer passes, was measured slower:
// single-target CTAs walk and stage for one target each.)  A range that fits nowhere sets the
// capacity error bit and records itself in the work counters' diagnostic slots.  Args must carry
// `L` (SmemLayout) and `work` (GroupWork).
constexpr int MAX_PAIR_PASSES = 14;
constexpr int PLAN_WORK_SLOT = 56;   // d_work[56]: work counter of the plan walk, [57] its pool counter

// Leaf-list capacity of the first pair pass (walk stacks hold at least 128 entries).
inline int first_pass_leaf_cap(const Ctx& c)
{
    return c.leaf_cap1 > 0 ? c.leaf_cap1 : (c.dim == 3 ? 256 : 96);
}

template <typename T>
PlanView<T> plan_view(Ctx& c)
{
    PlanView<T> v;
    v.plan = c.plan;
    v.plan_cap = c.plan_cap;
    v.leaves = c.pool_leaves;
    v.loff = reinterpret_cast<typename Vec4<T>::type*>(c.pool_loff);
    v.pool_cap = c.pool_cap;
    v.pool_count = c.d_work + PLAN_WORK_SLOT + 1;
    return v;
}

// Zeroes the plan walk's counters and launches it with four warps per block, as many blocks as fit.
template <class F>
void launch_plans(const void* kern, Ctx& c, size_t per_warp, F launch)
{
    cudaMemsetAsync(c.d_work + PLAN_WORK_SLOT, 0, 2 * sizeof(int), c.stream);
    const size_t smem = 4 * per_warp;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int nb = std::max(1, kernel_occupancy(kern, 128, smem));
    launch(nb * c.num_sms, smem);
}
constexpr int FAIL_INFO_SLOT = 48;   // d_work[48..52]: the last failing range
// d_err[1]: a capped tree build left a splittable node (read together with the status bits)
constexpr int GRID_BAR_SLOT = 61;    // d_work[61..62]: grid barrier of the fused level build (count, generation)
template <class Args>
void launch_pair_passes(Ctx& c, const void* kern, Args& a, int tcap, int elt4, int eltT,
                        void (*launch)(const void*, int, int, size_t, cudaStream_t, Args&),
                        const void* tpp_kern = nullptr,
                        void (*launch_tpp)(const void*, int, int, cudaStream_t, Args&) = nullptr);

// The largest source tile that fits the opt-in shared memory next to the walk capacities of the
// overflow pass.
inline int big_tile_cap(const Ctx& c, int gt, int elt4, int eltT, int stack_cap, int leaf_cap)
{
    const SmemLayout L0 = make_layout(gt, 0, elt4, eltT, stack_cap, leaf_cap);
    const size_t per = (size_t)elt4 + (size_t)eltT + sizeof(int) + (size_t)gt / 8 + (size_t)elt4 / 16;
    size_t cap = ((size_t)max_optin_smem(c) - L0.total - 64) / per;
    cap = cap / 32 * 32;
    if (cap > 16384) cap = 16384;
    return (int)cap;
}

template <class Args>
void launch_pair_passes(Ctx& c, const void* kern, Args& a, int tcap, int elt4, int eltT,
                        void (*launch)(const void*, int, int, size_t, cudaStream_t, Args&),
                        const void* tpp_kern,
                        void (*launch_tpp)(const void*, int, int, cudaStream_t, Args&))
{
    const int gt = c.group_threads;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_optin_smem(c));
    const int big = big_tile_cap(c, gt, elt4, eltT, 1024, 1024);
    int2* lists[2] = {c.d_ovf_list, c.d_ovf_list2};
    int halvings = 0;
    while ((1 << halvings) < gt) ++halvings;
    const int passes = std::min(MAX_PAIR_PASSES, 1 + (halvings + 1) + 2);
    // schedule (knob 28): 0 group passes down to single targets, 1 / 2 the first one / two group
    // passes and then the thread-per-particle kernel for the ranges left, 3 thread-per-particle only
    const int sched = tpp_kern ? c.pair_sched : 0;
    const int tpp_grid = tpp_kern ? std::max(1, kernel_occupancy(tpp_kern, 128, 0)) * c.num_sms : 0;
    if (sched == 3) {
        a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + 0, nullptr, nullptr, c.ovf_cap,
                           nullptr, nullptr, 0, 0, c.d_err, c.d_work + FAIL_INFO_SLOT};
        a.work.pieces = gt / 32;
        launch_tpp(tpp_kern, tpp_grid, 128, c.stream, a);
        return;
    }
    const int group_passes = sched == 1 ? 1 : sched == 2 ? 2 : passes;
    for (int pass = 0; pass < group_passes; ++pass) {
        int cap, stack_cap, leaf_cap, grid;
        const bool last_tier = pass >= passes - 2;
        if (pass == 0) {
            // walk capacities of the first pass: a 3D group's search box meets many more leaves
            // than a 2D one's (knob 27 overrides); the plan walk used the same
            cap = std::min(tcap, big);
            leaf_cap = first_pass_leaf_cap(c);
            stack_cap = std::max(128, leaf_cap);   // groups without a plan walk here
        }
        else if (!last_tier) {
            // walk capacities sized so that a 2D or 3D CTA of the doubled tile keeps a third block
            // per SM (1D trees with one particle per leaf need more leaf slots)
            cap = std::min(c.pass2_scale * tcap, big);
            stack_cap = 256;
            leaf_cap = c.dim == 1 ? 512 : 256;
        }
        else { cap = big; stack_cap = 1024; leaf_cap = 1024; }
        if (c.tile_limit > 0) cap = std::min(cap, c.tile_limit);
        a.L = make_layout(gt, cap, elt4, eltT, stack_cap, leaf_cap);
        grid = last_tier ? c.num_sms : std::max(1, kernel_occupancy(kern, gt, a.L.total)) * c.num_sms;
        // work counter 2 pass, produced-range count 2 pass + 1 (zeroed with the others)
        a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + 2 * pass,
                           pass == 0 ? nullptr : lists[(pass - 1) & 1],
                           pass == 0 ? nullptr : c.d_work + 2 * pass - 1, c.ovf_cap,
                           pass + 1 < passes ? lists[pass & 1] : nullptr,
                           c.d_work + 2 * pass + 1, c.ovf_cap, pass >= 1 ? 1 : 0, c.d_err,
                           c.d_work + FAIL_INFO_SLOT};
        launch(kern, grid, gt, a.L.total, c.stream, a);
    }
    if (sched == 1 || sched == 2) {
        const int last = group_passes - 1;
        a.work = GroupWork{c.g_begin, c.g_count, c.n_groups, c.d_work + 2 * group_passes, lists[last & 1],
                           c.d_work + 2 * last + 1, c.ovf_cap, nullptr, nullptr, 0, 0, c.d_err,
                           c.d_work + FAIL_INFO_SLOT};
        a.work.pieces = gt / 32;
        launch_tpp(tpp_kern, tpp_grid, 128, c.stream, a);
    }
}

}  // namespace sphgpu
