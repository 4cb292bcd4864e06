/*
 * sphgpu — C ABI of the GB300 (sm_103a) implementation of SPHCODE's per-step particle hot path.
 *
 * The reference has no FFI: its hot path is the sph::Module interface
 * (include/module.hpp:10-14: initialize(shared_ptr<SPHParameters>),
 * calculation(shared_ptr<Simulation>)) called by sph::Solver (src/solver.cpp:387-429).
 * Each entry point below is the device-side body of one of those calls, so a GPU Module
 * subclass is a drop-in that forwards its calculation() here (sphcode_gb300/cxx/gpu_modules.hpp
 * holds such subclasses).  Plain pointers and sizes only; no C++ or CUDA
 * types cross this boundary.  Every function returns an sphgpu_status code; no exception
 * crosses the ABI.
 *
 * Particle data at the boundary is in the caller's particle order (SPHParticle::id == index,
 * include/particle.hpp:30), FP64, vector fields interleaved per particle (x0 y0 z0 x1 ...).
 * Inside the library the particles live on the device as structure-of-arrays, reordered by
 * octree key; results are scattered back to the caller's order on download.
 */
#ifndef SPHGPU_H
#define SPHGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors sph::SPHParameters (include/parameters.hpp:20-79); JSON keys and defaults of
 * Solver::read_parameterfile (src/solver.cpp:193-298).  Same layout as the oracle's struct. */
typedef struct sphgpu_params {
    int    sph_type;          /* 0 ssph, 1 disph, 2 gsph                                       */
    int    kernel;            /* 0 cubic spline, 1 Wendland C4                                 */
    double cfl_sound;         /* cflSound                                                      */
    double cfl_force;         /* cflForce                                                      */
    double av_alpha;          /* avAlpha                                                       */
    int    use_balsara;       /* useBalsaraSwitch                                              */
    int    use_tdav;          /* useTimeDependentAV                                            */
    double alpha_max;         /* alphaMax                                                      */
    double alpha_min;         /* alphaMin                                                      */
    double epsilon_av;        /* epsilonAV                                                     */
    int    use_ac;            /* useArtificialConductivity                                     */
    double alpha_ac;          /* alphaAC                                                       */
    int    max_level;         /* maxTreeLevel                                                  */
    int    leaf_num;          /* leafParticleNumber                                            */
    int    neighbor_number;   /* neighborNumber                                                */
    double gamma;             /* gamma                                                         */
    int    iterative_sml;     /* iterativeSmoothingLength                                      */
    int    periodic;          /* periodic                                                      */
    double range_min[3];      /* rangeMin                                                      */
    double range_max[3];      /* rangeMax                                                      */
    int    use_gravity;       /* useGravity                                                    */
    double g_constant;        /* G                                                             */
    double theta;             /* theta                                                         */
    int    gsph_2nd_order;    /* use2ndOrderGSPH                                               */
} sphgpu_params;

typedef struct sphgpu_ctx sphgpu_ctx;

/* Arithmetic of the pair sums.  FP32_PAIR: pair terms in FP32 on offsets relative to the
 * target group's origin, per-particle totals Kahan-compensated; FP64 kept for absolute
 * positions/velocities/energies, the leapfrog, the smoothing-length Newton test, neighbour
 * membership decisions and global sums.  FP64: every pair term in FP64. */
enum sphgpu_precision { SPHGPU_FP32_PAIR = 0, SPHGPU_FP64 = 1 };

enum sphgpu_status {
    SPHGPU_OK = 0,
    SPHGPU_ERR_ARG = 1,          /* invalid argument / unsupported configuration               */
    SPHGPU_ERR_CUDA = 2,         /* CUDA runtime error (text in sphgpu_last_error)             */
    SPHGPU_ERR_NODE_POOL = 3,    /* octree needs more than 5 N nodes ("There is no free node",
                                    src/bhtree.cpp:179-181)                                    */
    SPHGPU_ERR_CAPACITY = 4,     /* a per-group walk stack, leaf list or source tile overflowed
                                    its capacity (the reference's neighbour list overflow is
                                    unchecked, src/pre_interaction.cpp:58)                     */
    SPHGPU_ERR_NOT_FINITE = 5,   /* NaN/Inf detected in a state field                          */
    SPHGPU_ERR_STATE = 6,        /* call order violated (e.g. forces before the tree)          */
    SPHGPU_ERR_NO_DEVICE = 7     /* no CUDA device / library built without a usable device     */
};

/* Field identifiers for sphgpu_set_field / sphgpu_get_field (SPHParticle members and the gsph
 * gradient arrays of src/solver.cpp:373-385).  Vector fields carry DIM doubles per particle;
 * GRAD_V carries DIM*DIM doubles per particle laid out [k][d] = d v_k / d x_d. */
enum sphgpu_field {
    SPHGPU_POS = 0, SPHGPU_VEL, SPHGPU_VEL_P, SPHGPU_ACC, SPHGPU_MASS, SPHGPU_DENS, SPHGPU_PRES,
    SPHGPU_ENE, SPHGPU_ENE_P, SPHGPU_DENE, SPHGPU_SML, SPHGPU_SOUND, SPHGPU_BALSARA,
    SPHGPU_ALPHA, SPHGPU_GRADH, SPHGPU_PHI, SPHGPU_NEIGHBOR, SPHGPU_GRAD_D, SPHGPU_GRAD_P,
    SPHGPU_GRAD_V, SPHGPU_NFIELDS
};

/* Simulation scalars (include/simulation.hpp:24-30). */
enum sphgpu_scalar { SPHGPU_TIME = 0, SPHGPU_DT = 1, SPHGPU_H_PER_V_SIG = 2 };

/* Byte offsets of SPHParticle members in a caller's array-of-structures (offsetof on the
 * caller's side), for the zero-repack upload/download used by the Module drop-in. */
typedef struct sphgpu_aos_layout {
    size_t stride;                           /* sizeof(SPHParticle)                            */
    long   pos, vel, vel_p, acc, mass, dens, pres, ene, ene_p, dene, sml, sound, balsara,
           alpha, gradh, phi;                /* offsets of FP64 members, -1 = absent          */
    long   neighbor;                         /* offset of the int member, -1 = absent         */
} sphgpu_aos_layout;

/* ---- lifetime ------------------------------------------------------------------------- */

/* One simulation of n particles in `dim` dimensions on the current CUDA device.
 * Replaces Simulation(param) + BHTree::initialize/resize (src/simulation.cpp:12-30,
 * src/bhtree.cpp:12-53) and each Module::initialize (e.g. src/pre_interaction.cpp:19-37). */
int sphgpu_create(const sphgpu_params* params, int dim, int n, int precision, sphgpu_ctx** out);

/* n_runs independent simulations of run_sizes[r] particles sharing one parameter set, advanced
 * together (each run keeps its own tree root, dt and time).  Particles of run r occupy the
 * index range [sum(run_sizes[0..r-1]), sum(run_sizes[0..r])) at the boundary.  No reference
 * counterpart (the reference runs one simulation per process). */
int sphgpu_create_batch(const sphgpu_params* params, int dim, int n_runs, const int* run_sizes,
                        int precision, sphgpu_ctx** out);

int sphgpu_destroy(sphgpu_ctx* ctx);

/* ---- data movement ---------------------------------------------------------------------- */

/* Host <-> device copies of one field in the caller's particle order (FP64; NEIGHBOR as
 * double).  Replace the reads/writes the modules do on Simulation::get_particles(). */
int sphgpu_set_field(sphgpu_ctx* ctx, int field, const double* host);
int sphgpu_get_field(sphgpu_ctx* ctx, int field, double* host);

/* Upload / download of a caller's std::vector<SPHParticle> storage in one contiguous copy;
 * only the members named in the layout are read or written back. */
int sphgpu_upload_aos(sphgpu_ctx* ctx, const void* base, const sphgpu_aos_layout* layout);
int sphgpu_download_aos(sphgpu_ctx* ctx, void* base, const sphgpu_aos_layout* layout);

/* Simulation::{set,get}_{time,dt,h_per_v_sig}; `run` selects the run of a batch (0 otherwise). */
int sphgpu_set_scalar(sphgpu_ctx* ctx, int which, int run, double value);
int sphgpu_get_scalar(sphgpu_ctx* ctx, int which, int run, double* value);

/* ---- the hot path ---------------------------------------------------------------------- */

/* Simulation::make_tree -> BHTree::make (src/simulation.cpp:37-40, src/bhtree.cpp:55-107). */
int sphgpu_make_tree(sphgpu_ctx* ctx);

/* PreInteraction::calculation for the context's SPH type (src/pre_interaction.cpp:39-169,
 * src/disph/d_pre_interaction.cpp:21-162, src/gsph/g_pre_interaction.cpp:27-144), including
 * the first-call initial_smoothing (:171-215) and the closing BHTree::set_kernel. */
int sphgpu_pre_interaction(sphgpu_ctx* ctx);

/* FluidForce::calculation (src/fluid_force.cpp:26-86, src/disph/d_fluid_force.cpp:26-86,
 * src/gsph/g_fluid_force.cpp:39-166). */
int sphgpu_fluid_force(sphgpu_ctx* ctx);

/* GravityForce::calculation with the tree (src/gravity_force.cpp:52-89,
 * src/bhtree.cpp:128-132,273-331); adds to the fluid acceleration. */
int sphgpu_gravity_force(sphgpu_ctx* ctx);

/* TimeStep::calculation (src/timestep.cpp:18-38). */
int sphgpu_timestep(sphgpu_ctx* ctx);

/* Solver::predict / Solver::correct (src/solver.cpp:431-474). */
int sphgpu_predict(sphgpu_ctx* ctx);
int sphgpu_correct(sphgpu_ctx* ctx);

/* Solver::initialize from the field start-up to the first force evaluation
 * (src/solver.cpp:392-414). */
int sphgpu_initialize(sphgpu_ctx* ctx);

/* n_steps of Solver::integrate + Simulation::update_time (src/solver.cpp:319-325,417-429),
 * replayed as one CUDA graph per step; the state stays on the device. */
int sphgpu_step(sphgpu_ctx* ctx, int n_steps);

/* Block until the context's stream is idle; returns any deferred device-side status. */
int sphgpu_synchronize(sphgpu_ctx* ctx);

/* ---- diagnostics and parity --------------------------------------------------------------- */

/* Neighbour sets for the current smoothing lengths in the caller's order: is_ij = 0 gives
 * {j : r_ij^2 < h_i^2}, is_ij = 1 gives {j : r_ij^2 < max(h_i^2, h_j^2)} — the sets of
 * exhaustive_search (src/exhaustive_search.cpp:11-42) and of the BHTree walk
 * (src/bhtree.cpp:234-270).  list holds cap ids per particle (unordered); list = NULL with
 * cap = 0 returns the counts only. */
int sphgpu_neighbors(sphgpu_ctx* ctx, int is_ij, int* counts, int* list, int cap);

/* Output::output_energy sums (src/output.cpp:66-90) plus momentum, summed in FP64:
 * out = {kinetic, thermal, potential, total, p_0 .. p_{DIM-1}} for run `run`. */
int sphgpu_energy(sphgpu_ctx* ctx, int run, double* out);

/* Tree shape: out[0] nodes (roots excluded), out[1] leaves, out[2+L] nodes at level L,
 * out[66+L] leaves at level L (130 ints). */
int sphgpu_tree_stats(sphgpu_ctx* ctx, int* out);

/* Target groups of the pair kernels formed by the last tree build (no reference counterpart: the
 * reference walks the tree once per particle): group_of[id] = group of the particle with caller
 * index id (groups numbered in key order), *n_groups = their number (n ints in group_of). */
int sphgpu_target_groups(sphgpu_ctx* ctx, int* group_of, int* n_groups);

/* Particles whose smoothing-length Newton iteration did not converge in the last
 * PreInteraction (the reference logs them, src/pre_interaction.cpp:277-280). */
int sphgpu_newton_failures(sphgpu_ctx* ctx, int* count);

/* Text of the last error on this context (or of the last failed create if ctx is NULL). */
const char* sphgpu_last_error(const sphgpu_ctx* ctx);

/* Kernel schedule knobs.  With autotune on (the default), sphgpu_initialize times
 * PreInteraction and FluidForce for candidate target-group sizes and tile capacities, then the
 * schedule family (knob 28) on the fastest of those, on the initial state and keeps the fastest;
 * setting 0, 3 or 10 explicitly turns the tuner off. */
/* Knobs:
 * which = 0 target-group size in warps, 1 FluidForce warps, 2 GravityForce warps,
 * 3 source-tile capacity (0 = automatic), 4 autotune on/off, 5 per-stage event timing on/off
 * (steps then run eagerly), 6 CUDA-graph replay of steps on/off; 7 (read only) kernel launches
 * in one captured step; 8, 9 (read only) target groups that overflowed into the large-capacity
 * pass in the last timed PreInteraction / FluidForce; 10 PreInteraction source-tile capacity
 * (0 = automatic; 3 then applies to FluidForce); 11 (read only) status bits raised by tuning
 * candidates that the tuner rejected; 12 tile of the second pair-kernel pass in multiples of the
 * first (1..8, default 2); 13..17 (read only) the last target range no pair-kernel pass could
 * fit: {first particle (key order), count, search radius x 1e9, leaves, overflow code};
 * 18 fixed time step on/off: with 1, sphgpu_step skips TimeStep and advances every run by the
 * dt last set with sphgpu_set_scalar(SPHGPU_SCALAR_DT) (the adjoint requires it);
 * 19 AoS record reuse on/off: with 1, sphgpu_download_aos takes the record members outside the
 * layout from the records of the last sphgpu_upload_aos (same stride) instead of copying the
 * caller's buffer to the device first — valid when the caller has not changed those members on
 * the host since that upload (the upload, calculate, download pattern of a Module);
 * 20, 21 (read only) the level limit of the last octree build, and the level limit of the
 * step builds without gravity (0: all key levels; raised by four whenever a build leaves a node
 * with more than leafParticleNumber particles unsplit at the limit);
 * 22 source-tile limit of every pair-kernel pass, the large-capacity passes included (0 = none;
 * a multiple of 32): targets whose sources do not fit make the stage return SPHGPU_ERR_CAPACITY
 * and record themselves in 13..17;
 * 23 octree node limit below the 5 N + runs pool (0 = none): a level whose children do not all
 * fit is left unsplit and the build returns SPHGPU_ERR_NODE_POOL ("There is no free node",
 * src/bhtree.cpp:179-181);
 * 24 tuner fault injection: bit k set makes the tuner's trial k (in trial order) count as having
 * raised the tile status bit, so that it is rejected (tests of the rejection path);
 * 25 work counters of the pair kernels on/off (sphgpu_pair_counters; off by default);
 * 27 leaf-list capacity of the first pair-kernel pass (0 = by dimension: 96 in 1D and 2D, 256 in
 * 3D; the walk stack holds at least as many entries);
 * 28 pair-kernel schedule: 0 target groups staged in shared memory, with later passes for the
 * ranges a pass cannot fit, halved down to single targets; 1 and 2 the first one or two group
 * passes, then the thread-per-particle kernel (each target walks the octree itself) for the
 * ranges left; 3 thread-per-particle only (PreInteraction and FluidForce alike; the tuner tries
 * all four on its chosen groups and tiles);
 * 29 tile staging of the group schedule by bulk asynchronous copies on/off: the particle records
 * of the walked leaves reach shared memory by one cp.async.bulk per leaf (mbarrier completion,
 * bounded waits) and are filtered in place, where they all fit the tile;
 * 30 target-group formation: 1 (default in 2D and 3D) the largest aligned key blocks (octree
 * cells and their halves, one key bit at a time) of at most 32 x knob 0 particles of one run,
 * compact in space; 0 (default in 1D, where such a chunk is an interval) fixed chunks of the key
 * order of that size, each split once where it straddles two distant cells.  Targets of a group
 * smaller than the CTA fill whole warps first; the other warps skip the group's pair work;
 * 31 group plans, bit 0 FluidForce, bit 1 PreInteraction (default 0): a walk kernel ahead of the
 * stage's first pass forms every group's box and leaf list with one warp per group, so that the
 * pass itself neither reduces the box nor walks the octree (groups without a plan walk there);
 * 32 octree levels in one cooperative launch on/off (default on in 2D and 3D): per level the child
 * placement and the children's split counts with one bounded grid-wide barrier, instead of two launches per level
 * (a barrier wait that runs out stops the build, the kernels that use the tree return at once and
 * the step returns SPHGPU_ERR_CUDA with the text in sphgpu_last_error);
 * 33 fault injection for the tests of that bounded wait: with 1, the next fused level build's
 * first block leaves without arriving at the first barrier, so the other blocks' wait runs out
 * (one build only; the knob then reads 0);
 * 34 key table: 0 off, 1 from 2^18 particles on (default), 2 always (reads 0 when a batch has too
 * many runs for its 64 MB): the first levels (ten for a single run, fewer for large batches) of
 * each run's octree-centre recursion replayed
 * once per tree build into a table that the key computation searches with integer comparisons
 * (the same keys, fewer FP64 additions);
 * 35 gravity work items: 1 fixed 32-particle chunks of each run's key order, one warp each
 * (default), 0 the pair kernels' target groups in pieces of 32 (partly filled warps). */
int sphgpu_set_tuning(sphgpu_ctx* ctx, int which, int value);
int sphgpu_get_tuning(sphgpu_ctx* ctx, int which, int* value);

/* Work counters of the pair kernels accumulated while knob 25 is on (no reference
 * counterpart; they feed the algorithmic work counts of the benchmark's roofline).  out[16]:
 * {0 PreInteraction targets, 1 sum of search-radius candidates |{j : r_ij < 1.2 h_guess}|,
 * 2 sum of Newton iterations, 3 sum of iterations x |{j : r_ij < h_i}|, 4 sum of neighbour counts
 * |{j : r_ij < h_i}|, 5 staged sources tested per PreInteraction target (summed), 6 the same for
 * FluidForce, 7 PreInteraction target ranges processed (all passes), 8 FluidForce ranges,
 * 9 GravityForce monopole terms, 10 GravityForce leaf particle pairs (self terms included),
 * 11..15 zero}.  reset != 0 zeroes them after the read. */
int sphgpu_pair_counters(sphgpu_ctx* ctx, unsigned long long* out, int reset);

/* Per-stage device time of the last sphgpu_step / stage call in milliseconds, measured with
 * CUDA events on the context's stream: out = {tree, pre, fluid, gravity, integrate}. */
int sphgpu_stage_times(sphgpu_ctx* ctx, double* out);

/* Benchmark helper (no reference counterpart): runs n_steps steps like sphgpu_step, each
 * bracketed by CUDA events on the context's stream; with flush_l2 != 0 a buffer of twice the
 * L2 size is overwritten before every step, outside the timed brackets.  *ms = sum of the
 * per-step device times. */
int sphgpu_bench_steps(sphgpu_ctx* ctx, int n_steps, int flush_l2, double* ms);

/* Calibration (no reference counterpart): sustained FP32 and FP64 FMA throughput of the current
 * device in TFLOP/s, the denominators of the pair kernels' compute rooflines. */
int sphgpu_measure_peaks(double* fp32_tflops, double* fp64_tflops);

/* ---- adjoint (reverse mode) of the SPH step (ssph, disph) -----------------------------------
 *
 * No counterpart in the reference: these entry points serve a gradient harness.  They
 * differentiate Solver::initialize and Solver::integrate (src/solver.cpp:392-474) with
 * PreInteraction (src/pre_interaction.cpp:39-169, smoothing length as the root of the Newton
 * equation, grad-h term, Balsara switch) and FluidForce (src/fluid_force.cpp:26-106), with
 * neighbour sets and the viscosity branch (v_ij . r_ij < 0) of the
 * forward pass.  Supported: sph_type ssph or disph (src/disph/d_pre_interaction.cpp:21-230,
 * src/disph/d_fluid_force.cpp:26-86), cubic spline or Wendland C4, no gravity, no
 * time-dependent viscosity, no artificial conductivity, iterative smoothing length, the fixed
 * time step (tuning knob 18), a single run.  Anything else returns SPHGPU_ERR_ARG.
 *
 * State vector (device pointer, caller's particle order, doubles):
 *   [x (n*dim) | v (n*dim) | u (n) | a (n*dim) | du/dt (n) | rho (n)]  = n * (3 dim + 3)
 * x, v, a interleaved per particle.  rho is the density the next PreInteraction starts its
 * smoothing-length guess from.  Adjoint vector (device pointer, caller's order, doubles):
 *   [xbar (n*dim) | vbar (n*dim) | ubar (n) | abar (n*dim) | dubar (n)]  = n * (3 dim + 2)
 * All pointers are device pointers; the work runs on the context's stream and the calls return
 * after it finished. */

/* Copy the integrator state out of / into the context (caller order). */
int sphgpu_get_state(sphgpu_ctx* ctx, double* state);
int sphgpu_set_state(sphgpu_ctx* ctx, const double* state);

/* Reverse one sphgpu_step.  The context must hold the state S_n the step started from
 * (sphgpu_set_state); adj holds the adjoint of S_{n+1} on entry and that of S_n on return.
 * dens_bar (may be NULL) is an extra adjoint of the density computed inside this step;
 * *alpha_bar (device double) accumulates the adjoint of avAlpha.  The call recomputes the step's
 * prediction, tree and PreInteraction, so the context holds that mid-step state afterwards. */
int sphgpu_adjoint_step(sphgpu_ctx* ctx, double* adj, const double* dens_bar, double* alpha_bar);

/* Reverse sphgpu_initialize.  The context must hold the initial fields (sphgpu_set_state with
 * the initial x, v, u and rho; a and du/dt are ignored).  adj holds the adjoint of S_0 on entry;
 * on return its x, v and u blocks hold the gradient with respect to the initial x, v and u, and
 * its a and du/dt blocks are zero. */
int sphgpu_adjoint_initialize(sphgpu_ctx* ctx, double* adj, const double* dens_bar, double* alpha_bar);

/* ---- allocation-free entry point ---------------------------------------------------------- */

/* Energy and momentum sums of sphgpu_energy over caller-owned device arrays, with no device
 * allocation at all.  No counterpart in the reference.  It is meant for callers that cannot
 * call cudaMalloc where they need the sums: host programs that own every byte of device memory
 * through a pool they reserved at start-up, and loops that must not stall the device (cudaMalloc
 * and cudaFree can synchronise it).
 *
 * Inputs are device pointers in the caller's particle order: mass[n], vel[n * dim] (interleaved
 * x0 y0 z0 x1 ...), ene[n] and phi[n] (phi may be NULL: potential 0).  out is a device pointer
 * to 4 + dim doubles {kinetic, thermal, potential, total, p_0 .. p_{dim-1}}, written on `stream`
 * (a cudaStream_t; NULL = the legacy default stream); the call returns once the work is queued.
 *
 * Scratch: a fixed file-scope device array of 4096 x 7 doubles (229,376 bytes) that every GPU
 * loading the library keeps until the process exits; hence n <= 33,554,432 (4096 chunks of 8192
 * particles), larger n returns SPHGPU_ERR_CAPACITY with the text in sphgpu_last_error(NULL).
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current, and looks it up again if the device's context has changed since (e.g.
 * after cudaDeviceReset); make that first call before any stream capture.  A CUDA error left
 * pending by the caller's earlier work is reported (SPHGPU_ERR_CUDA) and left pending; errors of
 * this call's own launches are cleared after they are reported.  All calls share the one
 * array: calls that may overlap on the GPU (different streams, or different host threads on the
 * same device) race on it and must be serialised by the caller. */
int sphgpu_energy_noalloc(int dim, int n, const double* mass, const double* vel, const double* ene,
                          const double* phi, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPHGPU_H */
