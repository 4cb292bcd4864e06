// Adjoint kernels instantiated for DIM = 3 (see adjoint_impl.cuh).
#include "adjoint_impl.cuh"

namespace sphgpu {

template <>
void launch_adjoint_dim<3>(Ctx& c, double* adj, const double* dens_bar, double* alpha_bar, bool initial)
{
    adjoint_dispatch<3>(c, adj, dens_bar, alpha_bar, initial);
}

}  // namespace sphgpu
