// Host build of the adjoint's kernel derivatives (sphcode_gb300/csrc/kderiv.cuh) for
// tests/test_kernel_derivs.py.
#include "kderiv.cuh"

template <int D, int K>
static double eval(int which, double r, double h)
{
    using KD = sphkd::KD<D, K, double>;
    switch (which) {
    case 0: return KD::w(r, h);
    case 1: return KD::w_h(r, h);
    case 2: return KD::w_hh(r, h);
    case 3: return KD::F(r, h);
    case 4: return KD::F_r(r, h);
    case 5: return KD::F_h(r, h);
    default: return 0.0;
    }
}

extern "C" double kd_eval(int D, int K, int which, double r, double h)
{
    if (K == 0) {
        if (D == 1) return eval<1, 0>(which, r, h);
        if (D == 2) return eval<2, 0>(which, r, h);
        return eval<3, 0>(which, r, h);
    }
    if (D == 2) return eval<2, 1>(which, r, h);
    return eval<3, 1>(which, r, h);
}
