// Shared device definitions of the sphgpu library: state layout, tree view, smoothing kernels,
// the reference's exact FP64 distance arithmetic, compensated sums and status bits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <type_traits>

#include "../../include/sphgpu.h"

namespace sphgpu {

constexpr int WARP = 32;
constexpr unsigned FULL = 0xffffffffu;
constexpr double PI = 3.14159265358979323846;
constexpr int MAX_LEVELS = 64;

// ------------------------------------------------------------------------------------------
// Device status word (bitwise OR of these; read by the host after a stage).
enum ErrBit : unsigned {
    ERR_NODE_POOL = 1u,
    ERR_STACK = 2u,
    ERR_LEAVES = 4u,
    ERR_TILE = 8u,
    ERR_LIST = 16u,
    ERR_GSTACK = 32u,
    ERR_NOT_FINITE = 64u,
    ERR_TIMEOUT = 128u,   // a bounded wait on an asynchronous copy ran out
};

// ------------------------------------------------------------------------------------------
// Particle state: structure of arrays in octree-key order.  Field slots of State::f.
enum Field {
    F_POS = 0,            // 3 components
    F_VEL = 3,
    F_VELP = 6,
    F_ACC = 9,
    F_MASS = 12,
    F_DENS = 13,
    F_PRES = 14,
    F_ENE = 15,
    F_ENEP = 16,
    F_DENE = 17,
    F_SML = 18,
    F_SOUND = 19,
    F_BALSARA = 20,
    F_ALPHA = 21,
    F_GRADH = 22,
    F_PHI = 23,
    F_GRADD = 24,         // 3
    F_GRADP = 27,         // 3
    F_GRADV = 30,         // 9, [k*3 + d]
    F_COUNT = 39
};

struct State {
    double* f[F_COUNT];   // nullptr for components beyond DIM / unused gsph arrays
    int* id;              // caller's index of the particle in each slot
    int* neighbor;        // PreInteraction neighbour count
    int* run;             // run of each slot (constant: runs are contiguous key ranges)
};

// Octree nodes, breadth-first: the roots of the runs are nodes 0..R-1; children of a node are
// consecutive.  first_child < 0 marks a leaf.
struct TreeView {
    const int* begin;
    const int* count;
    const int* first_child;
    const int* nchild;
    const double* center[3];
    const double* edge;
    const double* mass;
    const double* com[3];
    const double* ksize;
    // FP32 copies for the superset walk of the pair kernels: centres rounded to nearest, edge
    // and kernel size rounded up
    const float* cf[3];
    const float* ef;
    const float* kf;
    // one 64-byte record per node for the Barnes-Hut walk (built with gravity only)
    const struct GravNode* gn;
};

// The Barnes-Hut walk's view of a node, loaded with four 16-byte loads: the centre of mass as a
// two-float pair (hi = nearest float, lo = nearest float of the remainder), edge^2 and mass in
// FP32, the links, and the geometric centre's offset from the centre of mass (nearest float of
// the FP64 difference; leaf particles are stored relative to the geometric centre).
struct __align__(16) GravNode {
    float4 com;     // {com_hi.x, com_hi.y, com_hi.z, edge^2}
    float4 comlo;   // {com_lo.x, com_lo.y, com_lo.z, mass}
    int4 link;      // {first_child, nchild, begin, count}
    float4 cc;      // {centre - com (x, y, z), 0}
};

struct Periodic {
    int on;
    double lo[3], hi[3], len[3];
    float lenf[3];
    long long lo_o[3], hi_o[3];   // ordered-integer images of lo and hi (for compares off the FP64 pipe)
};

// ------------------------------------------------------------------------------------------
// Exact restatement of the reference's FP64 distance arithmetic (include/periodic.hpp:34-59,
// include/vector_type.hpp:140-150): each operation rounded to nearest, no contraction, the
// periodic image chosen among (d, d+L, d-L) with the first-smallest rule.
__device__ __forceinline__ double ref_axis(double xi, double xj, const Periodic& pb, int k)
{
    const double a = __dsub_rn(xi, xj);
    if (!pb.on) return a;
    const double b = __dadd_rn(a, pb.len[k]);
    const double c = __dsub_rn(a, pb.len[k]);
    const double fa = fabs(a), fb = fabs(b), fc = fabs(c);
    if (fa <= fb && fa <= fc) return a;
    if (fb <= fc && fb <= fa) return b;
    return c;
}

template <int D>
__device__ __forceinline__ double ref_r2(const double* xi, const double* xj, const Periodic& pb)
{
    const double d0 = ref_axis(xi[0], xj[0], pb, 0);
    double r2 = __dmul_rn(d0, d0);
#pragma unroll
    for (int k = 1; k < D; ++k) {
        const double d = ref_axis(xi[k], xj[k], pb, k);
        r2 = __dadd_rn(r2, __dmul_rn(d, d));
    }
    return r2;
}

// Minimum-image offset used for staging (any consistent image within half a box).
__device__ __forceinline__ double min_image(double d, const Periodic& pb, int k)
{
    if (!pb.on) return d;
    const double half = 0.5 * pb.len[k];
    if (d > half) d -= pb.len[k];
    else if (d < -half) d += pb.len[k];
    return d;
}
__device__ __forceinline__ float min_image_f(float d, const Periodic& pb, int k)
{
    if (!pb.on) return d;
    const float half = 0.5f * pb.lenf[k];
    if (d > half) d -= pb.lenf[k];
    else if (d < -half) d += pb.lenf[k];
    return d;
}

// ------------------------------------------------------------------------------------------
// Compensated (Kahan) accumulation for the FP32 form; plain accumulation in FP64.
template <typename T>
struct Sum {
    T s;
    __device__ __forceinline__ void zero() { s = T(0); }
    __device__ __forceinline__ void add(T x) { s += x; }
    __device__ __forceinline__ T get() const { return s; }
};
template <>
struct Sum<float> {
    float s, c;
    __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float x)
    {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double get() const { return (double)s - (double)c; }
};

// ------------------------------------------------------------------------------------------
// Smoothing kernels with support radius h (include/kernel/cubic_spline.hpp:27-51,
// include/kernel/wendland_kernel.hpp:30-48), templated on dimension and arithmetic type.
template <int D>
struct Sigma;
template <>
struct Sigma<1> { static constexpr double cubic = 2.0 / 3.0; static constexpr double c4 = 0.0; };
template <>
struct Sigma<2> { static constexpr double cubic = 10.0 / (7.0 * PI); static constexpr double c4 = 9.0 / PI; };
template <>
struct Sigma<3> { static constexpr double cubic = 1.0 / PI; static constexpr double c4 = 495.0 / (32.0 * PI); };

template <int D, typename T>
__device__ __forceinline__ T powD(T h)
{
    if (D == 1) return h;
    if (D == 2) return h * h;
    return h * h * h;
}

template <typename T>
__device__ __forceinline__ T pos_part(T x) { return x > T(0) ? x : T(0); }

// W(r, h), dW/dh and the scalar c of grad W = r_ij * c, given hinv = 1/h (and rinv = 1/r for
// the gradient), so that a pair costs multiplications only.
template <int D, int K, typename T>
struct Kern {
    static __device__ __forceinline__ T w(T r, T hinv)
    {
        if (K == 0) {
            const T hh = T(2) * hinv;                 // 1 / (h / 2)
            const T q = r * hh;
            const T a = pos_part(T(2) - q), b = pos_part(T(1) - q);
            return T(Sigma<D>::cubic) * powD<D>(hh) * (T(0.25) * (a * a * a) - b * b * b);
        } else {
            const T q = r * hinv;
            const T a = pos_part(T(1) - q);
            const T a2 = a * a;
            return T(Sigma<D>::c4) * powD<D>(hinv) * (a2 * a2 * a2) * (T(1) + T(6) * q + T(35.0 / 3.0) * q * q);
        }
    }
    static __device__ __forceinline__ T dhw(T r, T hinv)
    {
        if (K == 0) {
            const T hh = T(2) * hinv;
            const T q = r * hh;
            const T a = pos_part(T(2) - q), b = pos_part(T(1) - q);
            return T(0.5 * Sigma<D>::cubic) * (powD<D>(hh) * hh)
                 * (a * a * (T((3.0 + D) * 0.25) * q - T(0.5 * D)) + b * b * (T(-3.0 - D) * q + T(D)));
        } else {
            const T q = r * hinv;
            const T a = pos_part(T(1) - q);
            const T a2 = a * a;
            return T(-Sigma<D>::c4 / 3.0) * (powD<D>(hinv) * hinv) * (a2 * a2 * a)
                 * (T(3.0 * D) + T(15.0 * D) * q + T(-56.0 + 17.0 * D) * q * q - T(35.0 * (8.0 + D)) * (q * q * q));
        }
    }
    static __device__ __forceinline__ T dw_coef(T r, T rinv, T hinv)
    {
        if (K == 0) {
            if (r == T(0)) return T(0);             // the cubic spline's dw returns 0 at r = 0
            const T hh = T(2) * hinv;
            const T q = r * hh;
            const T a = pos_part(T(2) - q), b = pos_part(T(1) - q);
            return T(-Sigma<D>::cubic) * (powD<D>(hh) * hh) * rinv * (T(0.75) * a * a - T(3) * b * b);
        } else {
            const T q = r * hinv;
            const T a = pos_part(T(1) - q);
            const T a2 = a * a;
            return T(-56.0 / 3.0 * Sigma<D>::c4) * (powD<D>(hinv) * hinv * hinv) * (a2 * a2 * a) * (T(1) + T(5) * q);
        }
    }
};

// Bring the 128-byte line holding p into L1 (no register result, so it never stalls the warp).
__device__ __forceinline__ void prefetch_l1(const void* p)
{
    asm volatile("prefetch.global.L1 [%0];" :: "l"(p));
}

// 1/sqrt in T (the FP32 pair kernels are compiled with approximate division and square root).
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return 1.0 / sqrt(x); }

// Dimension constant A_D (src/pre_interaction.cpp:61-63).
template <int D>
__host__ __device__ constexpr double volume_const()
{
    return D == 1 ? 2.0 : D == 2 ? PI : 4.0 * PI / 3.0;
}

// ------------------------------------------------------------------------------------------
// Ordered-integer images of doubles for atomic min/max.
__device__ __forceinline__ long long dbl_to_ord(double x)
{
    long long i = __double_as_longlong(x);
    return i >= 0 ? i : (i ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double ord_to_dbl(long long i)
{
    return __longlong_as_double(i >= 0 ? i : (i ^ 0x7fffffffffffffffLL));
}
__host__ __device__ inline long long host_dbl_to_ord(double x)
{
    long long i;
    memcpy(&i, &x, 8);
    return i >= 0 ? i : (i ^ 0x7fffffffffffffffLL);
}

// ------------------------------------------------------------------------------------------
// Work counters of the pair kernels (sphgpu_pair_counters), collected only when asked for.
enum PairCounter : int {
    PC_PRE_TARGETS = 0,      // PreInteraction targets (non-initial passes)
    PC_PRE_CANDIDATES = 1,   // sum of |{j : r_ij < 1.2 h_guess}| (the search-radius candidates)
    PC_PRE_ITERS = 2,        // sum of Newton iterations run
    PC_PRE_ITER_PAIRS = 3,   // sum over targets of iterations x |{j : r_ij < h_i}|
    PC_PRE_PAIRS = 4,        // sum of |{j : r_ij < h_i}| (the neighbour counts)
    PC_PRE_TESTS = 5,        // staged sources tested per target, summed (candidate-mask tests)
    PC_FLUID_TESTS = 6,      // the same for FluidForce
    PC_PRE_GROUPS = 7,       // target ranges processed by PreInteraction (all passes)
    PC_FLUID_GROUPS = 8,     // target ranges processed by FluidForce (all passes)
    PC_GRAV_NODES = 9,       // Barnes-Hut monopole terms (accepted nodes), summed over targets
    PC_GRAV_PAIRS = 10,      // Barnes-Hut leaf particle pairs (self terms included), summed over targets
    PAIR_COUNTERS = 16
};

// The octree build of this step stopped early (a grid-barrier wait of the level build ran out):
// the kernels that use the tree return at once and the step reports the status.
__device__ __forceinline__ bool tree_failed(const unsigned* err)
{
    return (*(const volatile unsigned*)err & ERR_TIMEOUT) != 0u;
}

// Sound speed of a mirror record: inside a whole step (c_sound > 0) sqrt(c_sound u) from the
// predicted u, the value predict would have stored (the same FP64 expression in FP64 records;
// in FP32 records the IEEE FP32 root of the rounded product); otherwise the stored field.
template <typename T>
__device__ __forceinline__ T mirror_sound(const State& st, int i, double u, double c_sound)
{
    if (c_sound > 0.0) {
        if constexpr (std::is_same<T, float>::value) return __fsqrt_rn((float)(c_sound * u));
        else return sqrt(c_sound * u);
    }
    return (T)st.f[F_SOUND][i];
}

// Adds v over the 32 lanes of a converged warp into *p (lane 0 issues one atomic).
__device__ __forceinline__ void warp_count(unsigned long long* p, unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(p, v);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace sphgpu
