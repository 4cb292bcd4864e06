// Smoothing kernels with the derivatives the adjoint needs, usable on host and device.
//
// W(r, h) is the cubic spline (K = 0, support h, include/kernel/cubic_spline.hpp:27-51) or the
// Wendland C4 kernel (K = 1, include/kernel/wendland_kernel.hpp:30-48); grad W = r_ij F(r, h).
// With q = r / s (s = h / 2 for the cubic spline, s = h for C4) both are W = sigma s^-D omega(q),
// and the derivatives follow from omega, omega', omega'':
//   dW/dr  = r F,           F   = sigma s^-(D+2) omega'(q) / q
//   dW/dh  = -sigma s^-D chi(q) / h,                 chi = D omega + q omega'
//   d2W/dh2 = sigma s^-D [(D+1) chi + q chi'] / h^2,  chi' = (D+1) omega' + q omega''
//   dF/dr and dF/dh by differentiating F directly.
// The header has no CUDA dependency besides the SPH_HD qualifier, so a host build can check the
// derivatives against finite differences.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define SPH_HD __host__ __device__ __forceinline__
#else
#define SPH_HD inline
#endif

namespace sphkd {

constexpr double KD_PI = 3.14159265358979323846;

template <int D>
SPH_HD double sigma_cubic() { return D == 1 ? 2.0 / 3.0 : D == 2 ? 10.0 / (7.0 * KD_PI) : 1.0 / KD_PI; }
template <int D>
SPH_HD double sigma_c4() { return D == 1 ? 0.0 : D == 2 ? 9.0 / KD_PI : 495.0 / (32.0 * KD_PI); }

template <int D, typename T>
SPH_HD T ipow(T x) { return D == 1 ? x : D == 2 ? x * x : x * x * x; }

// omega, omega', omega'' of the kernel shape (q in kernel units)
template <int K, typename T>
SPH_HD void shape(T q, T& w0, T& w1, T& w2)
{
    if (K == 0) {
        const T a = q < T(2) ? T(2) - q : T(0);
        const T b = q < T(1) ? T(1) - q : T(0);
        w0 = T(0.25) * a * a * a - b * b * b;
        w1 = T(-0.75) * a * a + T(3) * b * b;
        w2 = T(1.5) * a - T(6) * b;
    } else {
        const T a = q < T(1) ? T(1) - q : T(0);
        const T a2 = a * a, a4 = a2 * a2;
        w0 = a4 * a2 * (T(1) + T(6) * q + T(35.0 / 3.0) * q * q);
        w1 = T(-56.0 / 3.0) * q * a4 * a * (T(1) + T(5) * q);
        w2 = T(-56.0 / 3.0) * a4 * (T(1) + T(4) * q - T(35) * q * q);
    }
}

// omega'/q without the 1/q singularity at q = 0 (cubic spline: returns 0 at r = 0 like the
// reference's dw; C4: the finite limit)
template <int K, typename T>
SPH_HD T shape_w1_over_q(T q)
{
    if (K == 0) {
        if (q == T(0)) return T(0);
        T w0, w1, w2;
        shape<K, T>(q, w0, w1, w2);
        return w1 / q;
    }
    const T a = q < T(1) ? T(1) - q : T(0);
    const T a2 = a * a;
    return T(-56.0 / 3.0) * a2 * a2 * a * (T(1) + T(5) * q);
}

template <int D, int K, typename T>
struct KD {
    static SPH_HD T sig() { return (T)(K == 0 ? sigma_cubic<D>() : sigma_c4<D>()); }
    static SPH_HD T scale(T h) { return K == 0 ? h * T(0.5) : h; }

    static SPH_HD T w(T r, T h)
    {
        const T s = scale(h), q = r / s;
        T w0, w1, w2;
        shape<K, T>(q, w0, w1, w2);
        return sig() / ipow<D>(s) * w0;
    }
    static SPH_HD T w_h(T r, T h)
    {
        const T s = scale(h), q = r / s;
        T w0, w1, w2;
        shape<K, T>(q, w0, w1, w2);
        return -sig() / ipow<D>(s) * (T(D) * w0 + q * w1) / h;
    }
    static SPH_HD T w_hh(T r, T h)
    {
        const T s = scale(h), q = r / s;
        T w0, w1, w2;
        shape<K, T>(q, w0, w1, w2);
        const T chi = T(D) * w0 + q * w1;
        const T chi1 = T(D + 1) * w1 + q * w2;
        return sig() / ipow<D>(s) * (T(D + 1) * chi + q * chi1) / (h * h);
    }
    // grad W = r_ij F
    static SPH_HD T F(T r, T h)
    {
        const T s = scale(h), q = r / s;
        return sig() / (ipow<D>(s) * s * s) * shape_w1_over_q<K, T>(q);
    }
    // dF/dr
    static SPH_HD T F_r(T r, T h)
    {
        const T s = scale(h), q = r / s;
        if (r == T(0)) return T(0);
        T w0, w1, w2;
        shape<K, T>(q, w0, w1, w2);
        // F = c w1(q) / q with c = sig s^-(D+2): dF/dr = c (w2 / q - w1 / q^2) / s
        return sig() / (ipow<D>(s) * s * s * s) * (w2 / q - w1 / (q * q));
    }
    // dF/dh
    static SPH_HD T F_h(T r, T h)
    {
        const T s = scale(h), q = r / s;
        // F = sig s^-(D+2) g(q), g = w1 / q; dF/dh = -sig s^-(D+2) [(D+2) g + q g'] / h,
        // q g' = w2 - w1 / q
        if (r == T(0)) {
            const T g = shape_w1_over_q<K, T>(q);
            return -sig() / (ipow<D>(s) * s * s) * T(D + 2) * g / h;
        }
        T w0, w1, w2;
        shape<K, T>(q, w0, w1, w2);
        const T g = w1 / q;
        return -sig() / (ipow<D>(s) * s * s) * (T(D + 2) * g + (w2 - g)) / h;
    }
};

}  // namespace sphkd
