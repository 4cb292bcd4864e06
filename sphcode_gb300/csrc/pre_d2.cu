// PreInteraction kernels instantiated for DIM = 2 (see pre_impl.cuh).
#include "pre_impl.cuh"

namespace sphgpu {

template <>
void launch_pre_dim<2>(Ctx& c, bool initial)
{
    const bool f32 = c.precision == SPHGPU_FP32_PAIR;
    const int type = c.p.sph_type;
    const int kern = c.p.kernel;
#define SPHGPU_PRE(T, TY, K) run_pre<2, T, TY, K>(c, initial)
    if (f32) {
        if (kern == 0) {
            if (type == 0) SPHGPU_PRE(float, 0, 0); else if (type == 1) SPHGPU_PRE(float, 1, 0); else SPHGPU_PRE(float, 2, 0);
        } else {
            if (type == 0) SPHGPU_PRE(float, 0, 1); else if (type == 1) SPHGPU_PRE(float, 1, 1); else SPHGPU_PRE(float, 2, 1);
        }
    } else {
        if (kern == 0) {
            if (type == 0) SPHGPU_PRE(double, 0, 0); else if (type == 1) SPHGPU_PRE(double, 1, 0); else SPHGPU_PRE(double, 2, 0);
        } else {
            if (type == 0) SPHGPU_PRE(double, 0, 1); else if (type == 1) SPHGPU_PRE(double, 1, 1); else SPHGPU_PRE(double, 2, 1);
        }
    }
#undef SPHGPU_PRE
}

}  // namespace sphgpu
