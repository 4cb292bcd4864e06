/*
 * Oracle interface — TEST INFRASTRUCTURE ONLY.
 *
 * Shared by the two CPU checkers of this repository:
 *   - oracle/sph_oracle.c     : a C restatement of SPHCODE's per-step hot path (the "port"),
 *                               built on every machine (including the GPU machine);
 *   - oracle/ref_harness.cpp  : a driver around the reference's own translation units
 *                               (src/bhtree.cpp, src/pre_interaction.cpp, ...), built only where
 *                               the reference sources are available.
 * Both export the same entry points, prefixed orcD_ (port) and refD_ (reference) with D = 1, 2, 3
 * the compile-time dimension (the reference fixes DIM at compile time, include/defines.hpp:5).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load these libraries.
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors sph::SPHParameters (include/parameters.hpp:20-79) as plain C.  Field order and types
 * are part of the ABI: the Python side declares the identical ctypes.Structure. */
typedef struct orc_params {
    int    sph_type;          /* 0 ssph, 1 disph, 2 gsph              (SPHType)               */
    int    kernel;            /* 0 cubic spline, 1 Wendland C4        (KernelType)            */
    double cfl_sound;         /* cflSound   (default 0.3)                                      */
    double cfl_force;         /* cflForce   (default 0.125)                                    */
    double av_alpha;          /* avAlpha    (default 1)                                        */
    int    use_balsara;       /* useBalsaraSwitch   (default true)                             */
    int    use_tdav;          /* useTimeDependentAV (default false)                            */
    double alpha_max;         /* alphaMax   (default 2)                                        */
    double alpha_min;         /* alphaMin   (default 0.1)                                      */
    double epsilon_av;        /* epsilonAV  (default 0.2)                                      */
    int    use_ac;            /* useArtificialConductivity (default false)                     */
    double alpha_ac;          /* alphaAC    (default 1)                                        */
    int    max_level;         /* maxTreeLevel        (default 20)                              */
    int    leaf_num;          /* leafParticleNumber  (default 1)                               */
    int    neighbor_number;   /* neighborNumber      (default 32)                              */
    double gamma;             /* gamma (required)                                              */
    int    iterative_sml;     /* iterativeSmoothingLength (default true)                       */
    int    periodic;          /* periodic (default false)                                      */
    double range_min[3];      /* rangeMin (first DIM entries used)                             */
    double range_max[3];      /* rangeMax                                                      */
    int    use_gravity;       /* useGravity (default false)                                    */
    double g_constant;        /* G      (default 1)                                            */
    double theta;             /* theta  (default 0.5)                                          */
    int    gsph_2nd_order;    /* use2ndOrderGSPH (default true)                                */
} orc_params;

/* Per-particle fields (SPHParticle, include/particle.hpp:8-33, plus the gsph extra arrays
 * registered in src/solver.cpp:373-385).  Vector fields hold DIM doubles per particle;
 * GRAD_V holds DIM*DIM doubles per particle laid out [k][d] = d(v_k)/d(x_d). */
enum orc_field {
    ORC_POS = 0, ORC_VEL, ORC_VEL_P, ORC_ACC, ORC_MASS, ORC_DENS, ORC_PRES, ORC_ENE, ORC_ENE_P,
    ORC_DENE, ORC_SML, ORC_SOUND, ORC_BALSARA, ORC_ALPHA, ORC_GRADH, ORC_PHI, ORC_NEIGHBOR,
    ORC_GRAD_D, ORC_GRAD_P, ORC_GRAD_V, ORC_NFIELDS
};

/* Simulation scalars (include/simulation.hpp:24-30). */
enum orc_scalar { ORC_TIME = 0, ORC_DT = 1, ORC_H_PER_V_SIG = 2 };

/* Stages of one Solver::integrate() (src/solver.cpp:417-429) plus the start-up field
 * initialisation of Solver::initialize (src/solver.cpp:392-404). */
enum orc_stage {
    ORC_STAGE_TIMESTEP = 0, ORC_STAGE_PREDICT, ORC_STAGE_MAKE_TREE, ORC_STAGE_PRE,
    ORC_STAGE_FLUID, ORC_STAGE_GRAVITY, ORC_STAGE_CORRECT, ORC_STAGE_INIT_FIELDS
};

/* Return codes. */
enum orc_status {
    ORC_OK = 0, ORC_ERR_ARG = 1, ORC_ERR_NODE_POOL = 2, ORC_ERR_NEIGHBOR_LIST = 3,
    ORC_ERR_EXCEPTION = 4
};

#define ORC_DECLARE(D)                                                                          \
    void*  orc##D##_create(const orc_params* p, int n);                                          \
    void   orc##D##_destroy(void* h);                                                            \
    int    orc##D##_set_field(void* h, int field, const double* src);                            \
    int    orc##D##_get_field(void* h, int field, double* dst);                                  \
    void   orc##D##_set_scalar(void* h, int which, double v);                                    \
    double orc##D##_get_scalar(void* h, int which);                                              \
    int    orc##D##_initialize(void* h);                                                         \
    int    orc##D##_stage(void* h, int stage);                                                   \
    int    orc##D##_step(void* h);                                                               \
    int    orc##D##_neighbors(void* h, int is_ij, int exhaustive, int* counts, int* list,        \
                              int cap);                                                          \
    int    orc##D##_tree_stats(void* h, int* out);                                               \
    void   orc##D##_energy(void* h, double* out);                                                \
    int    orc##D##_newton_failures(void* h);                                                    \
    void   orc##D##_set_threads(int n);

#ifdef __cplusplus
}
#endif
