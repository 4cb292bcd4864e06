// Streaming FP64 kernels: TimeStep (src/timestep.cpp:18-38), Solver::predict / correct
// (src/solver.cpp:431-474), the start-up field values (src/solver.cpp:392-404),
// Simulation::update_time (src/simulation.cpp:32-35) and the energy/momentum sums
// (src/output.cpp:66-90).  All per-run: in a batch each run has its own dt and time.
#include "context.cuh"

namespace sphgpu {

namespace {

constexpr int THREADS = 256;

// The force criterion dt_force_i = cflForce * sqrt(h_i / |a_i|) costs two FP64 square roots and
// one FP64 division per particle, and the FP64 pipe (1/64 of the FP32 rate) is what bounds the
// reduction.  The minimum is found exactly in two passes instead:
//  1. e_i = sqrt(h_i / |a_i|) in FP32 (IEEE division and square root, no contraction) and its
//     minimum per run.  Every FP32 rounding is at most 2^-24 relative and the sum of squares
//     has positive terms only, so |e_i / sqrt(h_i / |a_i|) - 1| < 4 * 2^-24 while h_i and the
//     largest |a_k| lie in [2^-60, 2^60] (no FP32 overflow, and a square below the normal range
//     only for components 2^30 times smaller than the largest); particles outside that range are
//     "wide" and always take the FP64 expression.
//  2. The FP64 expression only for the wide particles and those with e_i <= emin * (1 + 2^-12).
//     The FP64 values are within 2^-49 of cflForce * sqrt(h / |a|), so the particle of the FP64
//     minimum has an exact value at most 2^-48 above that of any other particle, its e_i at most
//     2^-20 above emin, and it is always evaluated: the minimum is the same FP64 number as the
//     minimum over all particles.
// A particle with all components of a_i zero keeps the empty value (|a_i| = 0 is skipped).
struct DtEstimate {
    float e;       // FP32 estimate of sqrt(h / |a|), +inf when a_i = 0
    bool wide;     // outside the estimate's range: evaluate in FP64
};

template <int D>
__device__ __forceinline__ DtEstimate dt_estimate(const State& st, int i)
{
    float a2 = 0.0f, amax = 0.0f;
    bool zero = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double a = st.f[F_ACC + k][i];
        zero = zero && (__double_as_longlong(a) << 1) == 0;
        const float af = (float)a;
        a2 += af * af;
        amax = fmaxf(amax, fabsf(af));
    }
    const float hf = (float)st.f[F_SML][i];
    constexpr float LO = 8.673617379884035e-19f, HI = 1.152921504606847e18f;   // 2^-60, 2^60
    DtEstimate d;
    d.wide = !zero && !(amax >= LO && amax <= HI && hf >= LO && hf <= HI);
    d.e = zero ? __int_as_float(0x7f800000) : sqrtf(hf / sqrtf(a2));
    return d;
}

// Minimum of v over a block's particles into dst[run]: a warp whose lanes share one run reduces
// by shuffles, the block's uniform warps of one run combine in shared memory and issue one atomic
// (one per block instead of one per warp: the per-warp atomics on one address serialised and
// took most of the kernels' time); lanes of warps that straddle runs add their own values.
template <typename V>
__device__ __forceinline__ void block_run_min(int r, V v, V* dst)
{
    __shared__ int s_run[THREADS / 32];
    __shared__ V s_val[THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned same = __match_any_sync(FULL, r);
    const bool uniform = same == FULL;
    if (uniform) {
        for (int o = 16; o > 0; o >>= 1) {
            const V u = __shfl_xor_sync(FULL, v, o);
            v = u < v ? u : v;
        }
    } else if (r >= 0) {
        atomicMin(&dst[r], v);
    }
    if (lane == 0) {
        s_run[w] = uniform ? r : -2;
        s_val[w] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        bool one = s_run[0] >= 0;
        V m = s_val[0];
        for (int q = 1; q < nw; ++q) {
            one = one && s_run[q] == s_run[0];
            m = s_val[q] < m ? s_val[q] : m;
        }
        if (one) {
            atomicMin(&dst[s_run[0]], m);
        } else {
            for (int q = 0; q < nw; ++q)
                if (s_run[q] >= 0) atomicMin(&dst[s_run[q]], s_val[q]);
        }
    }
}

template <int D>
__global__ void timestep_estimate_kernel(State st, int n, int* emin)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int v = 0x7f800000;   // +inf; non-negative floats order like their bit patterns
    int r = -1;
    if (i < n) {
        r = st.run[i];
        const DtEstimate d = dt_estimate<D>(st, i);
        if (!d.wide && d.e >= 0.0f) v = __float_as_int(d.e);   // NaN stays out
    }
    block_run_min<int>(r, v, emin);
}

template <int D>
__global__ void timestep_min_kernel(State st, int n, double cfl_force, const int* emin, long long* dtmin)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 1.7976931348623157e308;
    int r = -1;
    if (i < n) {
        r = st.run[i];
        const DtEstimate d = dt_estimate<D>(st, i);
        const float bound = __int_as_float(emin[r]) * 1.000244140625f;   // * (1 + 2^-12)
        if (d.wide || d.e <= bound) {
            double a2 = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) { const double a = st.f[F_ACC + k][i]; a2 += a * a; }
            const double a = sqrt(a2);
            if (a > 0.0) v = cfl_force * sqrt(st.f[F_SML][i] / a);
        }
    }
    // ordered-integer images: their minimum is the FP64 minimum (a NaN from the FP64 expression
    // has a positive image above every finite value, as fmin would leave it out)
    block_run_min<long long>(r, dbl_to_ord(v), dtmin);
}

// dt = min(cflSound * h_per_v_sig, dt_force); resets the minimum for the next call.
__global__ void timestep_final_kernel(int R, double cfl_sound, const long long* hvs,
                                      long long* dtmin, int* emin, double* dt)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const double ds = cfl_sound * ord_to_dbl(hvs[r]);
    const double df = ord_to_dbl(dtmin[r]);
    dt[r] = ds < df ? ds : df;
    dtmin[r] = dbl_to_ord(1.7976931348623157e308);
    emin[r] = 0x7f800000;
}

// SOUND false (inside a whole step): the sound speed is not stored here; the stages that follow
// form sqrt(c_sound u) from the predicted u in their mirror kernels, and correct stores it.
template <int D, bool SOUND>
__global__ void predict_kernel(State st, int n, const double* dt_run, double c_sound, Periodic pb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = dt_run[st.run[i]];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double v = st.f[F_VEL + k][i], a = st.f[F_ACC + k][i];
        const double vp = v + a * (0.5 * dt);
        st.f[F_VELP + k][i] = vp;
        double x = st.f[F_POS + k][i] + vp * dt;
        if (pb.on) {
            // x < lo and x > hi on the ordered-integer images (the same outcomes, NaN and -0.0
            // included, without two FP64 compares per axis)
            long long xb = __double_as_longlong(x);
            const bool nan = (xb & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
            if (xb == (long long)0x8000000000000000ULL) xb = 0;
            const long long xo = xb >= 0 ? xb : (xb ^ 0x7fffffffffffffffLL);
            if (!nan && xo < pb.lo_o[k]) x += pb.len[k];
            else if (!nan && xo > pb.hi_o[k]) x -= pb.len[k];
        }
        st.f[F_POS + k][i] = x;
        st.f[F_VEL + k][i] = v + a * dt;
    }
    const double u = st.f[F_ENE][i], du = st.f[F_DENE][i];
    st.f[F_ENEP][i] = u + du * (0.5 * dt);
    const double un = u + du * dt;
    st.f[F_ENE][i] = un;
    if (SOUND) st.f[F_SOUND][i] = sqrt(c_sound * un);
}

template <int D>
__global__ void correct_kernel(State st, int n, const double* dt_run, double c_sound)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = dt_run[st.run[i]];
#pragma unroll
    for (int k = 0; k < D; ++k)
        st.f[F_VEL + k][i] = st.f[F_VELP + k][i] + st.f[F_ACC + k][i] * (0.5 * dt);
    const double u = st.f[F_ENEP][i] + st.f[F_DENE][i] * (0.5 * dt);
    st.f[F_ENE][i] = u;
    st.f[F_SOUND][i] = sqrt(c_sound * u);
}

__global__ void init_fields_kernel(State st, int n, double alpha, double c_sound)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    st.f[F_ALPHA][i] = alpha;
    st.f[F_BALSARA][i] = 1.0;
    st.f[F_SOUND][i] = sqrt(c_sound * st.f[F_ENE][i]);
}

__global__ void update_time_kernel(int R, double* time, const double* dt)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < R) time[r] += dt[r];
}

// Energy and momentum of every run: one block per (run, chunk) slice writes partial sums, a
// second pass adds the partials of a run in a fixed order (deterministic).
constexpr int ESUM = 7;   // kinetic, thermal, potential, (unused), p_x, p_y, p_z
constexpr int ECHUNK = 8192;

template <int D>
__global__ void energy_partial_kernel(State st, const int* run_begin, int R, int chunks_per_run_max,
                                      double* partial)
{
    const int r = blockIdx.y;
    const int b0 = run_begin[r], e0 = run_begin[r + 1];
    const int chunk = blockIdx.x;
    const int b = b0 + chunk * ECHUNK, e = min(e0, b + ECHUNK);
    double s[ESUM] = {0, 0, 0, 0, 0, 0, 0};
    for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
        const double m = st.f[F_MASS][i];
        double v2 = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) { const double v = st.f[F_VEL + k][i]; v2 += v * v; s[4 + k] += m * v; }
        s[0] += 0.5 * m * v2;
        s[1] += m * st.f[F_ENE][i];
        s[2] += 0.5 * m * st.f[F_PHI][i];
    }
    __shared__ double red[ESUM][THREADS / 32];
#pragma unroll
    for (int q = 0; q < ESUM; ++q) {
        double v = s[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < ESUM) {
        double v = 0.0;
        for (int w = 0; w < THREADS / 32; ++w) v += red[threadIdx.x][w];
        partial[((size_t)r * chunks_per_run_max + chunk) * ESUM + threadIdx.x] = v;
    }
}

__global__ void energy_final_kernel(const int* run_begin, int R, int chunks_per_run_max,
                                    const double* partial, double* out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const int nch = (run_begin[r + 1] - run_begin[r] + ECHUNK - 1) / ECHUNK;
    double s[ESUM] = {0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < nch; ++c)
        for (int q = 0; q < ESUM; ++q) s[q] += partial[((size_t)r * chunks_per_run_max + c) * ESUM + q];
    out[r * ESUM + 0] = s[0];
    out[r * ESUM + 1] = s[1];
    out[r * ESUM + 2] = s[2];
    out[r * ESUM + 3] = s[0] + s[1] + s[2];
    out[r * ESUM + 4] = s[4];
    out[r * ESUM + 5] = s[5];
    out[r * ESUM + 6] = s[6];
}

}  // namespace

void launch_timestep(Ctx& c)
{
    const int g = ceil_div(c.n, THREADS);
    if (c.dim == 1) {
        timestep_estimate_kernel<1><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_emin);
        timestep_min_kernel<1><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.p.cfl_force, c.d_emin, c.d_dtmin);
    } else if (c.dim == 2) {
        timestep_estimate_kernel<2><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_emin);
        timestep_min_kernel<2><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.p.cfl_force, c.d_emin, c.d_dtmin);
    } else {
        timestep_estimate_kernel<3><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_emin);
        timestep_min_kernel<3><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.p.cfl_force, c.d_emin, c.d_dtmin);
    }
    timestep_final_kernel<<<ceil_div(c.R, 128), 128, 0, c.stream>>>(c.R, c.p.cfl_sound, c.d_hvs, c.d_dtmin,
                                                                     c.d_emin, c.d_dt);
}

void launch_predict(Ctx& c, bool store_sound)
{
    const int g = ceil_div(c.n, THREADS);
    const double cs = c.p.gamma * (c.p.gamma - 1.0);
    if (store_sound) {
        if (c.dim == 1) predict_kernel<1, true><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs, c.pb);
        else if (c.dim == 2) predict_kernel<2, true><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs, c.pb);
        else predict_kernel<3, true><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs, c.pb);
    } else {
        if (c.dim == 1) predict_kernel<1, false><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs, c.pb);
        else if (c.dim == 2) predict_kernel<2, false><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs, c.pb);
        else predict_kernel<3, false><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs, c.pb);
    }
}

void launch_correct(Ctx& c)
{
    const int g = ceil_div(c.n, THREADS);
    const double cs = c.p.gamma * (c.p.gamma - 1.0);
    if (c.dim == 1) correct_kernel<1><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs);
    else if (c.dim == 2) correct_kernel<2><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs);
    else correct_kernel<3><<<g, THREADS, 0, c.stream>>>(c.st, c.n, c.d_dt, cs);
}

void launch_init_fields(Ctx& c)
{
    init_fields_kernel<<<ceil_div(c.n, THREADS), THREADS, 0, c.stream>>>(
        c.st, c.n, c.p.av_alpha, c.p.gamma * (c.p.gamma - 1.0));
}

void launch_update_time(Ctx& c)
{
    update_time_kernel<<<ceil_div(c.R, 128), 128, 0, c.stream>>>(c.R, c.d_time, c.d_dt);
}

void launch_energy(Ctx& c, double* d_out)
{
    int maxc = 1;
    for (int r = 0; r < c.R; ++r) maxc = std::max(maxc, ceil_div(c.run_begin[r + 1] - c.run_begin[r], ECHUNK));
    dim3 grid(maxc, c.R);
    // partial buffer: reuse the stage buffer (sized at create for >= R * maxc * ESUM doubles)
    double* partial = c.d_sums;
    if (c.dim == 1) energy_partial_kernel<1><<<grid, THREADS, 0, c.stream>>>(c.st, c.d_run_begin, c.R, maxc, partial);
    else if (c.dim == 2) energy_partial_kernel<2><<<grid, THREADS, 0, c.stream>>>(c.st, c.d_run_begin, c.R, maxc, partial);
    else energy_partial_kernel<3><<<grid, THREADS, 0, c.stream>>>(c.st, c.d_run_begin, c.R, maxc, partial);
    energy_final_kernel<<<ceil_div(c.R, 128), 128, 0, c.stream>>>(c.d_run_begin, c.R, maxc, partial, d_out);
}

}  // namespace sphgpu
