/*
 * CPU restatement of SPHCODE's per-step particle hot path — TEST INFRASTRUCTURE (the oracle).
 *
 * This file is the checker for the CUDA library in sphcode_gb300/: it is never linked into the
 * product and the product never calls it.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it.
 *
 * It restates, in plain C99 + OpenMP, the reference's FP64 algorithms with the same arithmetic
 * (same formulas, same comparison conventions, same candidate lists sorted by distance) so that
 * its results agree with the reference modules to rounding.  Parity pin: tests/test_oracle_pin.py
 * compares every stage of this file with the reference's own translation units, driven by
 * oracle/ref_harness.cpp, and tests/golden/ holds fixtures produced by those reference modules.
 *
 * Compile-time dimension, like the reference (include/defines.hpp:5): build with -DDIM=1|2|3.
 * Exported symbols are prefixed orcD_ (see oracle/sph_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "sph_oracle.h"

#ifndef DIM
#error "compile with -DDIM=1, 2 or 3"
#endif

#if DIM == 1
#define NCHILD 2
#elif DIM == 2
#define NCHILD 4
#else
#define NCHILD 8
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define API(name) CAT(CAT(orc, DIM), CAT(_, name))

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Volume constant A_D of a unit sphere (src/pre_interaction.cpp:61-63). */
#if DIM == 1
static const double A_D = 2.0;
#elif DIM == 2
static const double A_D = M_PI;
#else
static const double A_D = 4.0 * M_PI / 3.0;
#endif

/* Neighbour-list capacity per particle: neighborNumber * 20 (include/defines.hpp:29,
 * src/pre_interaction.cpp:58). */
#define LIST_FACTOR 20

typedef struct { double x[DIM]; } vec;

static inline double dot(const double* a, const double* b)
{
    /* include/vector_type.hpp:140-150: a0*b0 + a1*b1 + a2*b2 evaluated left to right. */
    double s = a[0] * b[0];
    for (int k = 1; k < DIM; ++k) s = s + a[k] * b[k];
    return s;
}

static inline double sqr(double x) { return x * x; }

/* ------------------------------------------------------------------------------------------ */
/* Octree node: include/bhtree.hpp:19-53. Particles of a node form a singly linked list through
 * next[] (SPHParticle::next, include/particle.hpp:31). */
typedef struct {
    int    first;            /* first particle index, -1 = none */
    double mass;
    int    num;
    int    childs[NCHILD];   /* node pool index, -1 = none */
    double center[DIM];
    double m_center[DIM];
    double edge;
    int    level;
    double kernel_size;
    int    is_leaf;
} node_t;

typedef struct {
    orc_params p;
    int n;
    double *pos, *vel, *vel_p, *acc, *mass, *dens, *pres, *ene, *ene_p, *dene, *sml, *sound;
    double *balsara, *alpha, *gradh, *phi, *grad_d, *grad_p, *grad_v;
    int *neighbor, *next;
    double time, dt, h_per_v_sig;
    double kernel_ratio;
    int first_pre;
    int newton_fail;
    /* tree */
    node_t root;
    node_t* pool;
    int pool_size;
    int pool_used;
    int tree_error;
    /* periodic */
    double pmin[DIM], pmax[DIM], prange[DIM];
} sim_t;

/* ------------------------------------------------------------------------------------------ */
/* Periodic minimum image: include/periodic.hpp:34-59 (per axis the candidate among d, d+L, d-L
 * with the smallest magnitude, first match wins in the order (d, d+L, d-L)). */
static inline void rij(const sim_t* s, const double* ri, const double* rj, double* out)
{
    if (s->p.periodic) {
        for (int k = 0; k < DIM; ++k) {
            const double a = ri[k] - rj[k];
            const double b = a + s->prange[k];
            const double c = a - s->prange[k];
            const double fa = fabs(a), fb = fabs(b), fc = fabs(c);
            if (fa <= fb && fa <= fc) out[k] = a;
            else if (fb <= fc && fb <= fa) out[k] = b;
            else out[k] = c;
        }
    } else {
        for (int k = 0; k < DIM; ++k) out[k] = ri[k] - rj[k];
    }
}

/* include/periodic.hpp:61-72 */
static inline void periodic_apply(const sim_t* s, double* r)
{
    if (!s->p.periodic) return;
    for (int k = 0; k < DIM; ++k) {
        if (r[k] < s->pmin[k]) r[k] += s->prange[k];
        else if (r[k] > s->pmax[k]) r[k] -= s->prange[k];
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Smoothing kernels.  powh(h) = h^DIM (include/kernel/kernel_function.hpp:8-16). */
static inline double powh(double h)
{
#if DIM == 1
    return h;
#elif DIM == 2
    return h * h;
#else
    return h * h * h;
#endif
}

#if DIM == 1
static const double SIGMA_CUBIC = 2.0 / 3.0;
static const double SIGMA_C4 = 0.0;          /* undefined in 1D (wendland_kernel.hpp:15-16) */
#elif DIM == 2
static const double SIGMA_CUBIC = 10.0 / (7.0 * M_PI);
static const double SIGMA_C4 = 9.0 / M_PI;
#else
static const double SIGMA_CUBIC = 1.0 / M_PI;
static const double SIGMA_C4 = 495. / (32 * M_PI);
#endif

/* max(x, 0) written as 0.5 (x + |x|), the form the reference uses for the kernel cut-offs. */
static inline double pos_part(double x) { return 0.5 * (x + fabs(x)); }

/* Cubic spline M4 with support radius h (include/kernel/cubic_spline.hpp:27-51). */
static inline double cubic_w(double r, double h)
{
    const double hh = h * 0.5;
    const double q = r / hh;
    const double a = pos_part(2.0 - q), b = pos_part(1.0 - q);
    return SIGMA_CUBIC / powh(hh) * (0.25 * (a * a * a) - (b * b * b));
}
static inline double cubic_dw_coef(double r, double h)
{
    if (r == 0.0) return 0.0;
    const double hh = h * 0.5;
    const double q = r / hh;
    const double a = pos_part(2.0 - q), b = pos_part(1.0 - q);
    return -SIGMA_CUBIC / (powh(hh) * hh * r) * (0.75 * (a * a) - 3.0 * (b * b));
}
static inline double cubic_dhw(double r, double h)
{
    const double hh = h * 0.5;
    const double q = r / hh;
    const double a = pos_part(2.0 - q), b = pos_part(1.0 - q);
    return 0.5 * SIGMA_CUBIC / (powh(hh) * hh)
         * ((a * a) * ((3. + DIM) * 0.25 * q - 0.5 * DIM) + (b * b) * ((-3.0 - DIM) * q + DIM));
}

/* Wendland C4 (Dehnen & Aly 2012) with support h (include/kernel/wendland_kernel.hpp:30-48). */
static inline double c4_w(double r, double h)
{
    const double q = r / h;
    const double a = pos_part(1.0 - q);
    return SIGMA_C4 / powh(h) * (a * a * a * a * a * a) * (1.0 + 6.0 * q + 35.0 / 3.0 * q * q);
}
static inline double c4_dw_coef(double r, double h)
{
    const double q = r / h;
    const double a = pos_part(1.0 - q);
    return -56.0 / 3.0 * SIGMA_C4 / (powh(h) * sqr(h)) * (a * a * a * a * a) * (1.0 + 5.0 * q);
}
static inline double c4_dhw(double r, double h)
{
    const double q = r / h;
    const double a = pos_part(1.0 - q);
    return -SIGMA_C4 / (powh(h) * h * 3.0) * (a * a * a * a * a)
         * (3.0 * DIM + 15.0 * DIM * q + (-56.0 + 17.0 * DIM) * q * q - 35.0 * (8.0 + DIM) * (q * q * q));
}

static inline double kw(const sim_t* s, double r, double h)
{ return s->p.kernel == 0 ? cubic_w(r, h) : c4_w(r, h); }
static inline double kdhw(const sim_t* s, double r, double h)
{ return s->p.kernel == 0 ? cubic_dhw(r, h) : c4_dhw(r, h); }
static inline void kdw(const sim_t* s, const double* r_ij, double r, double h, double* out)
{
    const double c = s->p.kernel == 0 ? cubic_dw_coef(r, h) : c4_dw_coef(r, h);
    for (int k = 0; k < DIM; ++k) out[k] = r_ij[k] * c;
}

/* ------------------------------------------------------------------------------------------ */
/* Barnes-Hut octree (src/bhtree.cpp). */

static void node_clear(node_t* nd)
{
    nd->first = -1; nd->mass = 0.0; nd->num = 0;
    for (int c = 0; c < NCHILD; ++c) nd->childs[c] = -1;
    for (int k = 0; k < DIM; ++k) { nd->center[k] = 0.0; nd->m_center[k] = 0.0; }
    nd->edge = 0.0; nd->level = 0; nd->kernel_size = 0.0; nd->is_leaf = 0;
}

static inline node_t* node_at(sim_t* s, int idx) { return idx < 0 ? &s->root : &s->pool[idx]; }

/* BHNode::assign, src/bhtree.cpp:163-204: child index bit k set iff pos[k] > center[k]; a new
 * child's center is center[k] +/- edge/4 and its edge is edge/2. */
static void tree_assign(sim_t* s, node_t* nd, int ip)
{
    const double* pos = &s->pos[(size_t)ip * DIM];
    int index = 0;
    for (int k = 0; k < DIM; ++k) if (pos[k] > nd->center[k]) index |= (1 << k);
    int ci = nd->childs[index];
    if (ci < 0) {
        if (s->pool_used >= s->pool_size) { s->tree_error = ORC_ERR_NODE_POOL; return; }
        ci = s->pool_used++;
        nd->childs[index] = ci;
        node_t* ch = &s->pool[ci];
        node_clear(ch);
        ch->level = nd->level + 1;
        ch->edge = nd->edge * 0.5;
        for (int k = 0; k < DIM; ++k) {
            const double sgn = (index & (1 << k)) ? 1.0 : -1.0;
            ch->center[k] = nd->center[k] + sgn * nd->edge * 0.25;
        }
    }
    node_t* ch = &s->pool[ci];
    ch->num++;
    ch->mass += s->mass[ip];
    for (int k = 0; k < DIM; ++k) ch->m_center[k] += pos[k] * s->mass[ip];
    s->next[ip] = ch->first;
    ch->first = ip;
}

/* BHNode::create_tree, src/bhtree.cpp:136-161 (recursive, depth-first, children in index order;
 * a child is split further iff num > leafParticleNumber and the parent level < maxTreeLevel). */
static void tree_create(sim_t* s, int self)
{
    node_t* nd = node_at(s, self);
    for (int c = 0; c < NCHILD; ++c) nd->childs[c] = -1;
    int ip = nd->first;
    while (ip >= 0) {
        const int nx = s->next[ip];
        tree_assign(s, nd, ip);
        if (s->tree_error) return;
        ip = nx;
    }
    nd = node_at(s, self);
    const int level = nd->level;
    for (int c = 0; c < NCHILD; ++c) {
        const int ci = node_at(s, self)->childs[c];
        if (ci < 0) continue;
        node_t* ch = &s->pool[ci];
        for (int k = 0; k < DIM; ++k) ch->m_center[k] /= ch->mass;
        if (ch->num > s->p.leaf_num && level < s->p.max_level) {
            tree_create(s, ci);
            if (s->tree_error) return;
        } else {
            ch->is_leaf = 1;
        }
    }
}

/* BHTree::make, src/bhtree.cpp:55-107. */
static int tree_make(sim_t* s)
{
    node_t* r = &s->root;
    /* root_clear (include/bhtree.hpp:46-53) keeps center/edge/level */
    r->first = -1; r->mass = 0.0; r->num = 0;
    for (int k = 0; k < DIM; ++k) r->m_center[k] = 0.0;
    r->kernel_size = 0.0; r->is_leaf = 0;
    if (!s->p.periodic) {
        double lo[DIM], hi[DIM];
        for (int k = 0; k < DIM; ++k) { lo[k] = DBL_MAX; hi[k] = -DBL_MAX; }
        for (int i = 0; i < s->n; ++i)
            for (int k = 0; k < DIM; ++k) {
                const double x = s->pos[(size_t)i * DIM + k];
                if (lo[k] > x) lo[k] = x;
                if (hi[k] < x) hi[k] = x;
            }
        double l = 0.0;
        for (int k = 0; k < DIM; ++k) {
            r->center[k] = (hi[k] + lo[k]) * 0.5;
            const double range = hi[k] - lo[k];
            if (l < range) l = range;
        }
        r->edge = l;
    }
    for (int i = 0; i < s->n - 1; ++i) s->next[i] = i + 1;
    s->next[s->n - 1] = -1;
    r->first = 0;
    s->pool_used = 0;
    s->tree_error = 0;
    tree_create(s, -1);
    return s->tree_error;
}

/* BHNode::set_kernel, src/bhtree.cpp:206-232: per-node maximum smoothing length. */
static double tree_set_kernel(sim_t* s, int self)
{
    node_t* nd = node_at(s, self);
    double kernel = 0.0;
    if (nd->is_leaf) {
        for (int ip = nd->first; ip >= 0; ip = s->next[ip])
            if (s->sml[ip] > kernel) kernel = s->sml[ip];
    } else {
        for (int c = 0; c < NCHILD; ++c) {
            const int ci = nd->childs[c];
            if (ci < 0) continue;
            const double h = tree_set_kernel(s, ci);
            if (h > kernel) kernel = h;
        }
    }
    node_at(s, self)->kernel_size = kernel;
    return kernel;
}

typedef struct { double r2; int j; } cand_t;

static int cand_cmp(const void* a, const void* b)
{
    const double x = ((const cand_t*)a)->r2, y = ((const cand_t*)b)->r2;
    return (x < y) ? -1 : (x > y) ? 1 : 0;
}

/* BHNode::neighbor_search, src/bhtree.cpp:234-270: descend nodes whose Chebyshev distance from
 * the node center is <= edge/2 + h (h = max(h_i, kernel_size) when is_ij); in a leaf keep j with
 * r^2 < h^2. */
static void tree_search_rec(const sim_t* s, const node_t* nd, int i, int is_ij, cand_t* list,
                            int* n, int cap, int* overflow)
{
    const double* ri = &s->pos[(size_t)i * DIM];
    const double h = is_ij ? (s->sml[i] > nd->kernel_size ? s->sml[i] : nd->kernel_size) : s->sml[i];
    const double h2 = h * h;
    const double l2 = sqr(nd->edge * 0.5 + h);
    double d[DIM];
    rij(s, ri, nd->center, d);
    double dx2_max = sqr(d[0]);
    for (int k = 1; k < DIM; ++k) { const double t = sqr(d[k]); if (t > dx2_max) dx2_max = t; }
    if (!(dx2_max <= l2)) return;
    if (nd->is_leaf) {
        for (int jp = nd->first; jp >= 0; jp = s->next[jp]) {
            double r[DIM];
            rij(s, ri, &s->pos[(size_t)jp * DIM], r);
            const double r2 = dot(r, r);
            if (r2 < h2) {
                if (*n >= cap) { *overflow = 1; return; }
                list[*n].r2 = r2; list[*n].j = jp; ++*n;
            }
        }
    } else {
        for (int c = 0; c < NCHILD; ++c)
            if (nd->childs[c] >= 0)
                tree_search_rec(s, &s->pool[nd->childs[c]], i, is_ij, list, n, cap, overflow);
    }
}

/* src/exhaustive_search.cpp:11-42: all j with r^2 < h_i^2 (or < max(h_i^2, h_j^2) if is_ij). */
static int exhaustive(const sim_t* s, int i, int is_ij, cand_t* list, int cap, int* overflow)
{
    const double* ri = &s->pos[(size_t)i * DIM];
    const double hi2 = s->sml[i] * s->sml[i];
    int n = 0;
    for (int j = 0; j < s->n; ++j) {
        double r[DIM];
        rij(s, ri, &s->pos[(size_t)j * DIM], r);
        const double r2 = dot(r, r);
        const double hj2 = s->sml[j] * s->sml[j];
        const double k2 = is_ij ? (hi2 > hj2 ? hi2 : hj2) : hi2;
        if (r2 < k2) {
            if (n >= cap) { *overflow = 1; return n; }
            list[n].r2 = r2; list[n].j = j; ++n;
        }
    }
    qsort(list, n, sizeof(cand_t), cand_cmp);
    return n;
}

/* BHTree::neighbor_search, src/bhtree.cpp:114-126: walk, then sort the ids by r^2. */
static int search(const sim_t* s, int i, int is_ij, cand_t* list, int cap, int* overflow)
{
    int n = 0;
    tree_search_rec(s, &s->root, i, is_ij, list, &n, cap, overflow);
    qsort(list, n, sizeof(cand_t), cand_cmp);
    return n;
}

/* ------------------------------------------------------------------------------------------ */
/* Hernquist & Katz (1989) softened potential f and force g with e = h/2
 * (src/bhtree.cpp:273-299). */
static inline double hk_f(double r, double h)
{
    const double e = h * 0.5;
    const double u = r / e;
    if (u < 1.0) return (-0.5 * u * u * (1.0 / 3.0 - 3.0 / 20 * u * u + u * u * u / 20) + 1.4) / e;
    if (u < 2.0)
        return -1.0 / (15 * r) + (-u * u * (4.0 / 3.0 - u + 0.3 * u * u - u * u * u / 30) + 1.6) / e;
    return 1 / r;
}
static inline double hk_g(double r, double h)
{
    const double e = h * 0.5;
    const double u = r / e;
    if (u < 1.0) return (4.0 / 3.0 - 1.2 * u * u + 0.5 * u * u * u) / (e * e * e);
    if (u < 2.0)
        return (-1.0 / 15 + 8.0 / 3 * u * u * u - 3 * u * u * u * u + 1.2 * u * u * u * u * u
                - u * u * u * u * u * u / 6.0) / (r * r * r);
    return 1 / (r * r * r);
}

/* BHNode::calc_force, src/bhtree.cpp:301-331: open a node iff edge^2 > theta^2 |r_i - com|^2;
 * leaves are summed directly with the symmetrised softening, other nodes as monopoles. */
static void tree_force_rec(const sim_t* s, const node_t* nd, int i, double theta2, double G,
                           double* phi, double* acc)
{
    const double* ri = &s->pos[(size_t)i * DIM];
    const double l2 = nd->edge * nd->edge;
    double d[DIM];
    rij(s, ri, nd->m_center, d);
    const double d2 = dot(d, d);
    if (l2 > theta2 * d2) {
        if (nd->is_leaf) {
            for (int jp = nd->first; jp >= 0; jp = s->next[jp]) {
                double r[DIM];
                rij(s, ri, &s->pos[(size_t)jp * DIM], r);
                const double rr = sqrt(dot(r, r));
                *phi -= G * s->mass[jp] * (hk_f(rr, s->sml[i]) + hk_f(rr, s->sml[jp])) * 0.5;
                const double c = G * s->mass[jp] * (hk_g(rr, s->sml[i]) + hk_g(rr, s->sml[jp])) * 0.5;
                for (int k = 0; k < DIM; ++k) acc[k] -= r[k] * c;
            }
        } else {
            for (int c = 0; c < NCHILD; ++c)
                if (nd->childs[c] >= 0) tree_force_rec(s, &s->pool[nd->childs[c]], i, theta2, G, phi, acc);
        }
    } else {
        const double r_inv = 1.0 / sqrt(d2);
        *phi -= G * nd->mass * r_inv;
        const double c = G * nd->mass * (r_inv * r_inv * r_inv);
        for (int k = 0; k < DIM; ++k) acc[k] -= d[k] * c;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* PreInteraction (src/pre_interaction.cpp, src/disph/d_pre_interaction.cpp,
 * src/gsph/g_pre_interaction.cpp). */

static inline double powh_m1(double h)   /* h^(DIM-1), pre_interaction.cpp:217-225 */
{
#if DIM == 1
    (void)h; return 1;
#elif DIM == 2
    return h;
#else
    return h * h;
#endif
}

/* PreInteraction::newton_raphson (src/pre_interaction.cpp:227-283) for ssph/gsph (mass density,
 * b = m N/A) and disph::PreInteraction::newton_raphson (src/disph/d_pre_interaction.cpp:174-230,
 * number density, b = N/A).  Iterates over the distance-sorted candidate list with a break at
 * r >= h; stops when |dh| < 1e-4 (h + h_prev); falls back to the unscaled guess after 10. */
static double newton(sim_t* s, int i, const cand_t* list, int n_cand, int number_density, int* failed)
{
    double h_i = s->sml[i] / s->kernel_ratio;
    const double b = number_density ? s->p.neighbor_number / A_D : s->mass[i] * s->p.neighbor_number / A_D;
    const double eps = 1e-4;
    const double* ri = &s->pos[(size_t)i * DIM];
    for (int it = 0; it < 10; ++it) {
        const double h_b = h_i;
        double dens = 0.0, ddens = 0.0;
        for (int n = 0; n < n_cand; ++n) {
            const int j = list[n].j;
            double r_ij[DIM];
            rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
            const double r = sqrt(dot(r_ij, r_ij));
            if (r >= h_i) break;
            if (number_density) { dens += kw(s, r, h_i); ddens += kdhw(s, r, h_i); }
            else { dens += s->mass[j] * kw(s, r, h_i); ddens += s->mass[j] * kdhw(s, r, h_i); }
        }
        const double f = dens * powh(h_i) - b;
        const double df = ddens * powh(h_i) + DIM * dens * powh_m1(h_i);
        h_i -= f / df;
        if (fabs(h_i - h_b) < (h_i + h_b) * eps) return h_i;
    }
    *failed = 1;
    return s->sml[i] / s->kernel_ratio;
}

static inline double vec_norm(const double* v) { return sqrt(dot(v, v)); }

/* PreInteraction::initial_smoothing, src/pre_interaction.cpp:171-215. */
static int initial_smoothing(sim_t* s)
{
    const int cap = s->p.neighbor_number * LIST_FACTOR;
    int err = 0;
#pragma omp parallel
    {
        cand_t* list = (cand_t*)malloc(sizeof(cand_t) * (size_t)cap);
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < s->n; ++i) {
            s->sml[i] = pow(s->p.neighbor_number * s->mass[i] / (s->dens[i] * A_D), 1.0 / DIM);
            int ovf = 0;
            const int nn = search(s, i, 0, list, cap, &ovf);
            if (ovf) { err = ORC_ERR_NEIGHBOR_LIST; continue; }
            const double* ri = &s->pos[(size_t)i * DIM];
            double dens = 0.0;
            for (int n = 0; n < nn; ++n) {
                const int j = list[n].j;
                double r_ij[DIM];
                rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
                const double r = sqrt(dot(r_ij, r_ij));
                if (r >= s->sml[i]) break;
                dens += s->mass[j] * kw(s, r, s->sml[i]);
            }
            s->dens[i] = dens;
        }
        free(list);
    }
    return err;
}

static int pre_interaction(sim_t* s)
{
    if (s->first_pre) {
        const int e = initial_smoothing(s);
        if (e) return e;
        s->first_pre = 0;
    }
    const int type = s->p.sph_type;
    const int cap = s->p.neighbor_number * LIST_FACTOR;
    const double gamma = s->p.gamma;
    const double dt = s->dt;
    double hvs_min = DBL_MAX;
    int err = 0, fails = 0;
#pragma omp parallel
    {
        cand_t* list = (cand_t*)malloc(sizeof(cand_t) * (size_t)cap);
        double my_min = DBL_MAX;
#pragma omp for schedule(dynamic, 64) reduction(+ : fails)
        for (int i = 0; i < s->n; ++i) {
            s->sml[i] = pow(s->p.neighbor_number * s->mass[i] / (s->dens[i] * A_D), 1.0 / DIM) * s->kernel_ratio;
            int ovf = 0;
            const int n_tmp = search(s, i, 0, list, cap, &ovf);
            if (ovf) { err = ORC_ERR_NEIGHBOR_LIST; continue; }
            if (s->p.iterative_sml) {
                int failed = 0;
                s->sml[i] = newton(s, i, list, n_tmp, type == 1, &failed);
                fails += failed;
            }
            const double h = s->sml[i];
            const double* ri = &s->pos[(size_t)i * DIM];
            const double* vi = &s->vel[(size_t)i * DIM];
            double dens = 0.0, dh_dens = 0.0, pres_sum = 0.0, dh_pres = 0.0, n_i = 0.0, dh_n = 0.0;
            double v_sig_max = s->sound[i] * 2.0;
            int nnb = 0;
            for (int n = 0; n < n_tmp; ++n) {
                const int j = list[n].j;
                double r_ij[DIM];
                rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
                const double r = sqrt(dot(r_ij, r_ij));
                if (r >= h) break;
                ++nnb;
                const double w = kw(s, r, h);
                dens += s->mass[j] * w;
                if (type == 0) {
                    dh_dens += s->mass[j] * kdhw(s, r, h);
                } else if (type == 1) {
                    const double dhw = kdhw(s, r, h);
                    n_i += w;
                    pres_sum += s->mass[j] * s->ene[j] * w;
                    dh_pres += s->mass[j] * s->ene[j] * dhw;
                    dh_n += dhw;
                }
                if (i != j) {
                    double v_ij[DIM];
                    for (int k = 0; k < DIM; ++k) v_ij[k] = vi[k] - s->vel[(size_t)j * DIM + k];
                    const double v_sig = s->sound[i] + s->sound[j] - 3.0 * dot(r_ij, v_ij) / r;
                    if (v_sig > v_sig_max) v_sig_max = v_sig;
                }
            }
            s->dens[i] = dens;
            if (type == 0) {
                s->pres[i] = (gamma - 1.0) * dens * s->ene[i];
                s->gradh[i] = 1.0 / (1.0 + h / (DIM * dens) * dh_dens);
            } else if (type == 1) {
                s->pres[i] = (gamma - 1.0) * pres_sum;
                s->gradh[i] = h / (DIM * n_i) * dh_pres / (1.0 + h / (DIM * n_i) * dh_n);
            } else {
                s->pres[i] = (gamma - 1.0) * dens * s->ene[i];
            }
            s->neighbor[i] = nnb;
            const double hvs = h / v_sig_max;
            if (my_min > hvs) my_min = hvs;

            if (type == 2) {
                /* MUSCL gradients, src/gsph/g_pre_interaction.cpp:112-136 */
                if (!s->p.gsph_2nd_order) continue;
                double dd[DIM] = {0}, du[DIM] = {0}, dv[DIM][DIM];
                memset(dv, 0, sizeof(dv));
                for (int n = 0; n < nnb; ++n) {
                    const int j = list[n].j;
                    double r_ij[DIM], dw[DIM];
                    rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
                    const double r = sqrt(dot(r_ij, r_ij));
                    kdw(s, r_ij, r, h, dw);
                    for (int k = 0; k < DIM; ++k) {
                        dd[k] += dw[k] * s->mass[j];
                        du[k] += dw[k] * (s->mass[j] * (s->ene[j] - s->ene[i]));
                    }
                    for (int a = 0; a < DIM; ++a) {
                        const double c = s->mass[j] * (s->vel[(size_t)j * DIM + a] - vi[a]);
                        for (int k = 0; k < DIM; ++k) dv[a][k] += dw[k] * c;
                    }
                }
                const double rho_inv = 1.0 / s->dens[i];
                for (int k = 0; k < DIM; ++k) {
                    s->grad_d[(size_t)i * DIM + k] = dd[k];
                    s->grad_p[(size_t)i * DIM + k] = (dd[k] * s->ene[i] + du[k]) * (gamma - 1.0);
                }
                for (int a = 0; a < DIM; ++a)
                    for (int k = 0; k < DIM; ++k)
                        s->grad_v[((size_t)i * DIM + a) * DIM + k] = dv[a][k] * rho_inv;
                continue;
            }

            /* Artificial viscosity switches, src/pre_interaction.cpp:115-161 and
             * src/disph/d_pre_interaction.cpp:106-154. */
            const double wfac = (type == 1) ? 1.0 : 0.0;
            (void)wfac;
            if (s->p.use_balsara && DIM != 1) {
                double div_v = 0.0;
#if DIM == 2
                double rot_v = 0.0;
#else
                double rot_v[3] = {0.0, 0.0, 0.0};
#endif
                for (int n = 0; n < nnb; ++n) {
                    const int j = list[n].j;
                    double r_ij[DIM], dw[DIM], v_ij[DIM];
                    rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
                    const double r = sqrt(dot(r_ij, r_ij));
                    kdw(s, r_ij, r, h, dw);
                    for (int k = 0; k < DIM; ++k) v_ij[k] = vi[k] - s->vel[(size_t)j * DIM + k];
                    const double wj = (type == 1) ? s->mass[j] * s->ene[j] : s->mass[j];
                    div_v -= wj * dot(v_ij, dw);
#if DIM == 2
                    rot_v += (v_ij[0] * dw[1] - v_ij[1] * dw[0]) * wj;
#elif DIM == 3
                    rot_v[0] += (v_ij[1] * dw[2] - v_ij[2] * dw[1]) * wj;
                    rot_v[1] += (v_ij[2] * dw[0] - v_ij[0] * dw[2]) * wj;
                    rot_v[2] += (v_ij[0] * dw[1] - v_ij[1] * dw[0]) * wj;
#endif
                }
                double rot_abs;
                if (type == 1) {
                    const double p_inv = (gamma - 1.0) / s->pres[i];
                    div_v *= p_inv;
#if DIM == 2
                    rot_v *= p_inv;
#elif DIM == 3
                    for (int k = 0; k < 3; ++k) rot_v[k] *= p_inv;
#endif
                } else {
                    div_v /= s->dens[i];
#if DIM == 2
                    rot_v /= s->dens[i];
#elif DIM == 3
                    for (int k = 0; k < 3; ++k) rot_v[k] /= s->dens[i];
#endif
                }
#if DIM == 2
                rot_abs = fabs(rot_v);
#elif DIM == 3
                rot_abs = sqrt(rot_v[0] * rot_v[0] + rot_v[1] * rot_v[1] + rot_v[2] * rot_v[2]);
#else
                rot_abs = 0.0;
#endif
                s->balsara[i] = fabs(div_v) / (fabs(div_v) + rot_abs + 1e-4 * s->sound[i] / h);
                if (s->p.use_tdav) {
                    const double tau_inv = s->p.epsilon_av * s->sound[i] / h;
                    const double sdiv = -div_v > 0.0 ? -div_v : 0.0;
                    const double dalpha = (-(s->alpha[i] - s->p.alpha_min) * tau_inv
                                           + sdiv * (s->p.alpha_max - s->alpha[i])) * dt;
                    s->alpha[i] += dalpha;
                }
            } else if (s->p.use_tdav) {
                double div_v = 0.0;
                for (int n = 0; n < nnb; ++n) {
                    const int j = list[n].j;
                    double r_ij[DIM], dw[DIM], v_ij[DIM];
                    rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
                    const double r = sqrt(dot(r_ij, r_ij));
                    kdw(s, r_ij, r, h, dw);
                    for (int k = 0; k < DIM; ++k) v_ij[k] = vi[k] - s->vel[(size_t)j * DIM + k];
                    const double wj = (type == 1) ? s->mass[j] * s->ene[j] : s->mass[j];
                    div_v -= wj * dot(v_ij, dw);
                }
                if (type == 1) div_v *= (gamma - 1.0) / s->pres[i];
                else div_v /= s->dens[i];
                const double tau_inv = s->p.epsilon_av * s->sound[i] / h;
                const double s_i = -div_v > 0.0 ? -div_v : 0.0;
                s->alpha[i] = (s->alpha[i] + dt * tau_inv * s->p.alpha_min + s_i * dt * s->p.alpha_max)
                            / (1.0 + dt * tau_inv + s_i * dt);
            }
        }
#pragma omp critical
        { if (hvs_min > my_min) hvs_min = my_min; }
        free(list);
    }
    s->h_per_v_sig = hvs_min;
    s->newton_fail += fails;
    tree_set_kernel(s, -1);
    return err;
}

/* ------------------------------------------------------------------------------------------ */
/* FluidForce (src/fluid_force.cpp:26-116, src/disph/d_fluid_force.cpp:26-86,
 * src/gsph/g_fluid_force.cpp:28-199). */

/* Monaghan (1997) signal-velocity viscosity, src/fluid_force.cpp:89-106 */
static inline double art_visc(const sim_t* s, int i, int j, const double* r_ij, double r_abs)
{
    double v_ij[DIM];
    for (int k = 0; k < DIM; ++k) v_ij[k] = s->vel[(size_t)i * DIM + k] - s->vel[(size_t)j * DIM + k];
    const double vr = dot(v_ij, r_ij);
    if (vr < 0) {
        const double alpha = 0.5 * (s->alpha[i] + s->alpha[j]);
        const double balsara = 0.5 * (s->balsara[i] + s->balsara[j]);
        const double w_ij = vr / r_abs;
        const double v_sig = s->sound[i] + s->sound[j] - 3.0 * w_ij;
        const double rho_ij_inv = 2.0 / (s->dens[i] + s->dens[j]);
        return -0.5 * balsara * alpha * v_sig * w_ij * rho_ij_inv;
    }
    return 0;
}

/* Price (2008) / Wadsley et al. (2008) conductivity, src/fluid_force.cpp:108-116 */
static inline double art_cond(const sim_t* s, int i, int j, const double* r_ij, double r_abs,
                              const double* dw_ij)
{
    double v_sig;
    if (s->p.use_gravity) {
        double v_ij[DIM];
        for (int k = 0; k < DIM; ++k) v_ij[k] = s->vel[(size_t)i * DIM + k] - s->vel[(size_t)j * DIM + k];
        v_sig = fabs(dot(v_ij, r_ij) / r_abs);
    } else {
        v_sig = sqrt(2.0 * fabs(s->pres[i] - s->pres[j]) / (s->dens[i] + s->dens[j]));
    }
    return s->p.alpha_ac * s->mass[j] * v_sig * (s->ene[i] - s->ene[j]) * dot(dw_ij, r_ij) / r_abs;
}

/* van Leer (1979) limiter, src/gsph/g_fluid_force.cpp:28-36 */
static inline double limiter(double dq1, double dq2)
{
    const double p = dq1 * dq2;
    if (p <= 0) return 0.0;
    return 2.0 * p / (dq1 + dq2);
}

/* HLL solver with Roe-averaged wave speeds, src/gsph/g_fluid_force.cpp:168-199.
 * q = (velocity along e_ij, density, pressure, sound speed). */
static inline void hll(const double* left, const double* right, double* pstar, double* vstar)
{
    const double u_l = left[0], rho_l = left[1], p_l = left[2], c_l = left[3];
    const double u_r = right[0], rho_r = right[1], p_r = right[2], c_r = right[3];
    const double roe_l = sqrt(rho_l), roe_r = sqrt(rho_r);
    const double roe_inv = 1.0 / (roe_l + roe_r);
    const double u_t = (roe_l * u_l + roe_r * u_r) * roe_inv;
    const double c_t = (roe_l * c_l + roe_r * c_r) * roe_inv;
    const double a = u_l - c_l, b = u_t - c_t;
    const double s_l = a < b ? a : b;
    const double c = u_r + c_r, d = u_t + c_t;
    const double s_r = c > d ? c : d;
    const double c1 = rho_l * (s_l - u_l);
    const double c2 = rho_r * (s_r - u_r);
    const double c3 = 1.0 / (c1 - c2);
    const double c4 = p_l - u_l * c1;
    const double c5 = p_r - u_r * c2;
    *vstar = (c5 - c4) * c3;
    *pstar = (c1 * c5 - c2 * c4) * c3;
}

static int fluid_force(sim_t* s)
{
    const int type = s->p.sph_type;
    const int cap = s->p.neighbor_number * LIST_FACTOR;
    const double gamma = s->p.gamma;
    const double dt = s->dt;
    int err = 0;
#pragma omp parallel
    {
        cand_t* list = (cand_t*)malloc(sizeof(cand_t) * (size_t)cap);
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < s->n; ++i) {
            int ovf = 0;
            const int nn = search(s, i, 1, list, cap, &ovf);
            if (ovf) { err = ORC_ERR_NEIGHBOR_LIST; continue; }
            const double* ri = &s->pos[(size_t)i * DIM];
            const double* vi = &s->vel[(size_t)i * DIM];
            const double h_i = s->sml[i];
            double acc[DIM] = {0};
            double dene = 0.0;
            /* per-i constants of the three formulations */
            const double p_per_rho2_i = s->pres[i] / sqr(s->dens[i]);
            const double gradh_i = s->gradh[i];
            const double gamma2_u_i = sqr(gamma - 1.0) * s->ene[i];
            const double gamma2_u_per_pres_i = gamma2_u_i / s->pres[i];
            const double m_u_inv = 1.0 / (s->mass[i] * s->ene[i]);
            const double rho2_inv_i = 1.0 / sqr(s->dens[i]);
            for (int n = 0; n < nn; ++n) {
                const int j = list[n].j;
                double r_ij[DIM];
                rij(s, ri, &s->pos[(size_t)j * DIM], r_ij);
                const double r = sqrt(dot(r_ij, r_ij));
                const double hmax = h_i > s->sml[j] ? h_i : s->sml[j];
                if (r >= hmax || r == 0.0) continue;
                const double* vj = &s->vel[(size_t)j * DIM];
                double dw_i[DIM], dw_j[DIM], dw_ij[DIM], v_ij[DIM];
                kdw(s, r_ij, r, h_i, dw_i);
                kdw(s, r_ij, r, s->sml[j], dw_j);
                if (type == 2) {
                    const double r_inv = 1.0 / r;
                    double e_ij[DIM];
                    for (int k = 0; k < DIM; ++k) e_ij[k] = r_ij[k] * r_inv;
                    const double ve_i = dot(vi, e_ij), ve_j = dot(vj, e_ij);
                    double vstar, pstar;
                    if (s->p.gsph_2nd_order) {
                        /* MUSCL reconstruction, Murante et al. (2011),
                         * src/gsph/g_fluid_force.cpp:98-135 */
                        double right[4], left[4];
                        const double delta_i = 0.5 * (1.0 - s->sound[i] * dt * r_inv);
                        const double delta_j = 0.5 * (1.0 - s->sound[j] * dt * r_inv);
                        const double dv_ij = ve_i - ve_j;
                        double dv_i[DIM], dv_j[DIM];
                        for (int a = 0; a < DIM; ++a) {
                            dv_i[a] = dot(&s->grad_v[((size_t)i * DIM + a) * DIM], e_ij);
                            dv_j[a] = dot(&s->grad_v[((size_t)j * DIM + a) * DIM], e_ij);
                        }
                        const double dve_i = dot(dv_i, e_ij) * r;
                        const double dve_j = dot(dv_j, e_ij) * r;
                        right[0] = ve_i - limiter(dv_ij, dve_i) * delta_i;
                        left[0] = ve_j + limiter(dv_ij, dve_j) * delta_j;
                        const double dd_ij = s->dens[i] - s->dens[j];
                        const double dd_i = dot(&s->grad_d[(size_t)i * DIM], e_ij) * r;
                        const double dd_j = dot(&s->grad_d[(size_t)j * DIM], e_ij) * r;
                        right[1] = s->dens[i] - limiter(dd_ij, dd_i) * delta_i;
                        left[1] = s->dens[j] + limiter(dd_ij, dd_j) * delta_j;
                        const double dp_ij = s->pres[i] - s->pres[j];
                        const double dp_i = dot(&s->grad_p[(size_t)i * DIM], e_ij) * r;
                        const double dp_j = dot(&s->grad_p[(size_t)j * DIM], e_ij) * r;
                        right[2] = s->pres[i] - limiter(dp_ij, dp_i) * delta_i;
                        left[2] = s->pres[j] + limiter(dp_ij, dp_j) * delta_j;
                        right[3] = sqrt(gamma * right[2] / right[1]);
                        left[3] = sqrt(gamma * left[2] / left[1]);
                        hll(left, right, &pstar, &vstar);
                    } else {
                        const double right[4] = {ve_i, s->dens[i], s->pres[i], s->sound[i]};
                        const double left[4] = {ve_j, s->dens[j], s->pres[j], s->sound[j]};
                        hll(left, right, &pstar, &vstar);
                    }
                    const double rho2_inv_j = 1.0 / sqr(s->dens[j]);
                    double f[DIM];
                    for (int k = 0; k < DIM; ++k)
                        f[k] = dw_i[k] * (s->mass[j] * pstar * rho2_inv_i) + dw_j[k] * (s->mass[j] * pstar * rho2_inv_j);
                    double vdiff[DIM];
                    for (int k = 0; k < DIM; ++k) { acc[k] -= f[k]; vdiff[k] = e_ij[k] * vstar - vi[k]; }
                    dene -= dot(f, vdiff);
                    continue;
                }
                for (int k = 0; k < DIM; ++k) { dw_ij[k] = (dw_i[k] + dw_j[k]) * 0.5; v_ij[k] = vi[k] - vj[k]; }
                const double pi_ij = art_visc(s, i, j, r_ij, r);
                const double dene_ac = s->p.use_ac ? art_cond(s, i, j, r_ij, r, dw_ij) : 0.0;
                if (type == 0) {
                    const double ci = s->mass[j] * (p_per_rho2_i * gradh_i + 0.5 * pi_ij);
                    const double cj = s->mass[j] * (s->pres[j] / sqr(s->dens[j]) * s->gradh[j] + 0.5 * pi_ij);
                    for (int k = 0; k < DIM; ++k) acc[k] -= dw_i[k] * ci + dw_j[k] * cj;
                    dene += s->mass[j] * p_per_rho2_i * gradh_i * dot(v_ij, dw_i)
                          + 0.5 * s->mass[j] * pi_ij * dot(v_ij, dw_ij) + dene_ac;
                } else {
                    const double f_ij = 1.0 - gradh_i / (s->mass[j] * s->ene[j]);
                    const double f_ji = 1.0 - s->gradh[j] * m_u_inv;
                    const double u_per_pres_j = s->ene[j] / s->pres[j];
                    const double ci = s->mass[j] * (gamma2_u_per_pres_i * s->ene[j] * f_ij + 0.5 * pi_ij);
                    const double cj = s->mass[j] * (gamma2_u_i * u_per_pres_j * f_ji + 0.5 * pi_ij);
                    for (int k = 0; k < DIM; ++k) acc[k] -= dw_i[k] * ci + dw_j[k] * cj;
                    dene += s->mass[j] * gamma2_u_per_pres_i * s->ene[j] * f_ij * dot(v_ij, dw_i)
                          + 0.5 * s->mass[j] * pi_ij * dot(v_ij, dw_ij) + dene_ac;
                }
            }
            for (int k = 0; k < DIM; ++k) s->acc[(size_t)i * DIM + k] = acc[k];
            s->dene[i] = dene;
        }
        free(list);
    }
    return err;
}

/* GravityForce::calculation, src/gravity_force.cpp:52-89 (tree path), adds to acc. */
static int gravity_force(sim_t* s)
{
    if (!s->p.use_gravity) return 0;
    const double theta2 = s->p.theta * s->p.theta;
    const double G = s->p.g_constant;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < s->n; ++i) {
        double phi = 0.0;
        double* acc = &s->acc[(size_t)i * DIM];
        tree_force_rec(s, &s->root, i, theta2, G, &phi, acc);
        s->phi[i] = phi;
    }
    return 0;
}

/* TimeStep::calculation, src/timestep.cpp:18-38. */
static void timestep(sim_t* s)
{
    double dt_min = DBL_MAX;
    for (int i = 0; i < s->n; ++i) {
        const double a = vec_norm(&s->acc[(size_t)i * DIM]);
        if (a > 0.0) {
            const double d = s->p.cfl_force * sqrt(s->sml[i] / a);
            if (d < dt_min) dt_min = d;
        }
    }
    const double dt_sound = s->p.cfl_sound * s->h_per_v_sig;
    s->dt = dt_sound < dt_min ? dt_sound : dt_min;
}

/* Solver::predict / Solver::correct, src/solver.cpp:431-474 (kick-drift-kick leapfrog). */
static void predict(sim_t* s)
{
    const double dt = s->dt;
    const double c_sound = s->p.gamma * (s->p.gamma - 1.0);
#pragma omp parallel for
    for (int i = 0; i < s->n; ++i) {
        double* x = &s->pos[(size_t)i * DIM];
        double* v = &s->vel[(size_t)i * DIM];
        double* vp = &s->vel_p[(size_t)i * DIM];
        const double* a = &s->acc[(size_t)i * DIM];
        for (int k = 0; k < DIM; ++k) vp[k] = v[k] + a[k] * (0.5 * dt);
        s->ene_p[i] = s->ene[i] + s->dene[i] * (0.5 * dt);
        for (int k = 0; k < DIM; ++k) { x[k] += vp[k] * dt; v[k] += a[k] * dt; }
        s->ene[i] += s->dene[i] * dt;
        s->sound[i] = sqrt(c_sound * s->ene[i]);
        periodic_apply(s, x);
    }
}
static void correct(sim_t* s)
{
    const double dt = s->dt;
    const double c_sound = s->p.gamma * (s->p.gamma - 1.0);
#pragma omp parallel for
    for (int i = 0; i < s->n; ++i) {
        for (int k = 0; k < DIM; ++k)
            s->vel[(size_t)i * DIM + k] = s->vel_p[(size_t)i * DIM + k] + s->acc[(size_t)i * DIM + k] * (0.5 * dt);
        s->ene[i] = s->ene_p[i] + s->dene[i] * (0.5 * dt);
        s->sound[i] = sqrt(c_sound * s->ene[i]);
    }
}

/* Start-up field values, src/solver.cpp:392-404. */
static void init_fields(sim_t* s)
{
    const double c_sound = s->p.gamma * (s->p.gamma - 1.0);
    for (int i = 0; i < s->n; ++i) {
        s->alpha[i] = s->p.av_alpha;
        s->balsara[i] = 1.0;
        s->sound[i] = sqrt(c_sound * s->ene[i]);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Exported entry points. */

static double** field_ptr(sim_t* s, int f, int* width)
{
    *width = 1;
    switch (f) {
    case ORC_POS: *width = DIM; return &s->pos;
    case ORC_VEL: *width = DIM; return &s->vel;
    case ORC_VEL_P: *width = DIM; return &s->vel_p;
    case ORC_ACC: *width = DIM; return &s->acc;
    case ORC_MASS: return &s->mass;
    case ORC_DENS: return &s->dens;
    case ORC_PRES: return &s->pres;
    case ORC_ENE: return &s->ene;
    case ORC_ENE_P: return &s->ene_p;
    case ORC_DENE: return &s->dene;
    case ORC_SML: return &s->sml;
    case ORC_SOUND: return &s->sound;
    case ORC_BALSARA: return &s->balsara;
    case ORC_ALPHA: return &s->alpha;
    case ORC_GRADH: return &s->gradh;
    case ORC_PHI: return &s->phi;
    case ORC_GRAD_D: *width = DIM; return &s->grad_d;
    case ORC_GRAD_P: *width = DIM; return &s->grad_p;
    case ORC_GRAD_V: *width = DIM * DIM; return &s->grad_v;
    default: return NULL;
    }
}

void* API(create)(const orc_params* p, int n)
{
    if (!p || n <= 0) return NULL;
    sim_t* s = (sim_t*)calloc(1, sizeof(sim_t));
    s->p = *p;
    s->n = n;
    for (int f = 0; f < ORC_NFIELDS; ++f) {
        int w;
        double** fp = field_ptr(s, f, &w);
        if (fp) *fp = (double*)calloc((size_t)n * w, sizeof(double));
    }
    s->neighbor = (int*)calloc((size_t)n, sizeof(int));
    s->next = (int*)calloc((size_t)n, sizeof(int));
    s->kernel_ratio = p->iterative_sml ? 1.2 : 1.0;   /* src/pre_interaction.cpp:30-35 */
    s->first_pre = 1;
    s->time = 0.0;
    s->dt = 0.0;
    for (int k = 0; k < DIM; ++k) {
        s->pmin[k] = p->range_min[k];
        s->pmax[k] = p->range_max[k];
        s->prange[k] = s->pmax[k] - s->pmin[k];
    }
    /* BHTree::initialize, src/bhtree.cpp:12-40 */
    node_clear(&s->root);
    s->root.level = 1;
    if (p->periodic) {
        double l = 0.0;
        for (int k = 0; k < DIM; ++k) {
            s->root.center[k] = (s->pmax[k] + s->pmin[k]) * 0.5;
            if (l < s->prange[k]) l = s->prange[k];
        }
        s->root.edge = l;
    }
    /* BHTree::resize, node pool of 5 N (src/bhtree.cpp:42-53) */
    s->pool_size = 5 * n;
    s->pool = (node_t*)calloc((size_t)s->pool_size, sizeof(node_t));
    return s;
}

void API(destroy)(void* h)
{
    sim_t* s = (sim_t*)h;
    if (!s) return;
    for (int f = 0; f < ORC_NFIELDS; ++f) {
        int w;
        double** fp = field_ptr(s, f, &w);
        if (fp) free(*fp);
    }
    free(s->neighbor); free(s->next); free(s->pool); free(s);
}

int API(set_field)(void* h, int f, const double* src)
{
    sim_t* s = (sim_t*)h;
    if (f == ORC_NEIGHBOR) {
        for (int i = 0; i < s->n; ++i) s->neighbor[i] = (int)src[i];
        return 0;
    }
    int w;
    double** fp = field_ptr(s, f, &w);
    if (!fp) return ORC_ERR_ARG;
    memcpy(*fp, src, sizeof(double) * (size_t)s->n * w);
    return 0;
}

int API(get_field)(void* h, int f, double* dst)
{
    sim_t* s = (sim_t*)h;
    if (f == ORC_NEIGHBOR) {
        for (int i = 0; i < s->n; ++i) dst[i] = s->neighbor[i];
        return 0;
    }
    int w;
    double** fp = field_ptr(s, f, &w);
    if (!fp) return ORC_ERR_ARG;
    memcpy(dst, *fp, sizeof(double) * (size_t)s->n * w);
    return 0;
}

void API(set_scalar)(void* h, int which, double v)
{
    sim_t* s = (sim_t*)h;
    if (which == ORC_TIME) s->time = v;
    else if (which == ORC_DT) s->dt = v;
    else if (which == ORC_H_PER_V_SIG) s->h_per_v_sig = v;
}

double API(get_scalar)(void* h, int which)
{
    sim_t* s = (sim_t*)h;
    if (which == ORC_TIME) return s->time;
    if (which == ORC_DT) return s->dt;
    return s->h_per_v_sig;
}

int API(stage)(void* h, int stage)
{
    sim_t* s = (sim_t*)h;
    switch (stage) {
    case ORC_STAGE_TIMESTEP: timestep(s); return 0;
    case ORC_STAGE_PREDICT: predict(s); return 0;
    case ORC_STAGE_MAKE_TREE: return tree_make(s);
    case ORC_STAGE_PRE: return pre_interaction(s);
    case ORC_STAGE_FLUID: return fluid_force(s);
    case ORC_STAGE_GRAVITY: return gravity_force(s);
    case ORC_STAGE_CORRECT: correct(s); return 0;
    case ORC_STAGE_INIT_FIELDS: init_fields(s); return 0;
    default: return ORC_ERR_ARG;
    }
}

/* Solver::initialize from the field start-up to the first force evaluation
 * (src/solver.cpp:392-414). */
int API(initialize)(void* h)
{
    sim_t* s = (sim_t*)h;
    init_fields(s);
    int e = tree_make(s);
    if (e) return e;
    if ((e = pre_interaction(s))) return e;
    if ((e = fluid_force(s))) return e;
    return gravity_force(s);
}

/* Solver::integrate + Simulation::update_time (src/solver.cpp:417-429, 324). */
int API(step)(void* h)
{
    sim_t* s = (sim_t*)h;
    timestep(s);
    predict(s);
    int e = tree_make(s);
    if (e) return e;
    if ((e = pre_interaction(s))) return e;
    if ((e = fluid_force(s))) return e;
    if ((e = gravity_force(s))) return e;
    correct(s);
    s->time += s->dt;
    return 0;
}

/* Neighbour lists with the current smoothing lengths: the BHTree walk (exhaustive = 0) or the
 * O(N^2) exhaustive_search (exhaustive = 1); is_ij selects the Fluid criterion.  Lists are
 * sorted by distance; list has cap entries per particle. */
int API(neighbors)(void* h, int is_ij, int exh, int* counts, int* list, int cap)
{
    sim_t* s = (sim_t*)h;
    int err = 0;
#pragma omp parallel
    {
        cand_t* c = (cand_t*)malloc(sizeof(cand_t) * (size_t)cap);
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < s->n; ++i) {
            int ovf = 0;
            const int nn = exh ? exhaustive(s, i, is_ij, c, cap, &ovf) : search(s, i, is_ij, c, cap, &ovf);
            if (ovf) err = ORC_ERR_NEIGHBOR_LIST;
            counts[i] = nn;
            if (list)   /* NULL: counts only */
                for (int k = 0; k < nn; ++k) list[(size_t)i * cap + k] = c[k].j;
        }
        free(c);
    }
    return err;
}

static void stats_rec(const sim_t* s, const node_t* nd, int* out)
{
    for (int c = 0; c < NCHILD; ++c) {
        const int ci = nd->childs[c];
        if (ci < 0) continue;
        const node_t* ch = &s->pool[ci];
        out[0]++;
        if (ch->level < 64) out[2 + ch->level]++;
        if (ch->is_leaf) { out[1]++; if (ch->level < 64) out[66 + ch->level]++; }
        else stats_rec(s, ch, out);
    }
}

/* Tree shape summary: out[0] nodes (root excluded), out[1] leaves, out[2+L] nodes at level L,
 * out[66+L] leaves at level L (L < 64). */
int API(tree_stats)(void* h, int* out)
{
    sim_t* s = (sim_t*)h;
    memset(out, 0, sizeof(int) * 130);
    stats_rec(s, &s->root, out);
    return 0;
}

/* Output::output_energy sums (src/output.cpp:66-90) plus total momentum:
 * out = {kinetic, thermal, potential, total, p_0 .. p_{DIM-1}}. */
void API(energy)(void* h, double* out)
{
    sim_t* s = (sim_t*)h;
    double ek = 0.0, et = 0.0, ep = 0.0, mom[DIM] = {0};
    for (int i = 0; i < s->n; ++i) {
        const double* v = &s->vel[(size_t)i * DIM];
        ek += 0.5 * s->mass[i] * dot(v, v);
        et += s->mass[i] * s->ene[i];
        ep += 0.5 * s->mass[i] * s->phi[i];
        for (int k = 0; k < DIM; ++k) mom[k] += s->mass[i] * v[k];
    }
    out[0] = ek; out[1] = et; out[2] = ep; out[3] = ek + et + ep;
    for (int k = 0; k < DIM; ++k) out[4 + k] = mom[k];
}

int API(newton_failures)(void* h) { return ((sim_t*)h)->newton_fail; }

void API(set_threads)(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
