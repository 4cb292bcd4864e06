// FluidForce kernels instantiated for DIM = 2 (see fluid_impl.cuh).
#include "fluid_impl.cuh"

namespace sphgpu {

template <>
void launch_fluid_dim<2>(Ctx& c)
{
    const bool f32 = c.precision == SPHGPU_FP32_PAIR;
    const int type = c.p.sph_type;
    const int kern = c.p.kernel;
#define SPHGPU_FLUID(T, TY, K) run_fluid<2, T, TY, K>(c)
    if (f32) {
        if (kern == 0) {
            if (type == 0) SPHGPU_FLUID(float, 0, 0); else if (type == 1) SPHGPU_FLUID(float, 1, 0); else SPHGPU_FLUID(float, 2, 0);
        } else {
            if (type == 0) SPHGPU_FLUID(float, 0, 1); else if (type == 1) SPHGPU_FLUID(float, 1, 1); else SPHGPU_FLUID(float, 2, 1);
        }
    } else {
        if (kern == 0) {
            if (type == 0) SPHGPU_FLUID(double, 0, 0); else if (type == 1) SPHGPU_FLUID(double, 1, 0); else SPHGPU_FLUID(double, 2, 0);
        } else {
            if (type == 0) SPHGPU_FLUID(double, 0, 1); else if (type == 1) SPHGPU_FLUID(double, 1, 1); else SPHGPU_FLUID(double, 2, 1);
        }
    }
#undef SPHGPU_FLUID
}

}  // namespace sphgpu
