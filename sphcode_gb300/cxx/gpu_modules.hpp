// GPU drop-ins for the reference's sph::Module implementations (include/module.hpp:10-14).
//
// Each class forwards Module::calculation() to the sphgpu C-ABI (include/sphgpu.h) on one GPU:
//   sph::gpu::PreInteraction  replaces sph::PreInteraction / disph:: / gsph::PreInteraction
//                             (src/pre_interaction.cpp:39-169, src/disph/d_pre_interaction.cpp:21-162,
//                             src/gsph/g_pre_interaction.cpp:27-144), BHTree::set_kernel included;
//   sph::gpu::FluidForce      replaces sph::FluidForce / disph:: / gsph::FluidForce
//                             (src/fluid_force.cpp:26-116, src/disph/d_fluid_force.cpp:26-86,
//                             src/gsph/g_fluid_force.cpp:39-166);
//   sph::gpu::GravityForce    replaces sph::GravityForce (src/gravity_force.cpp:52-89).
// The SPH type, kernel and every other setting come from the SPHParameters given to
// initialize(), as in the reference.  The three modules of one Simulation share a Device, which
// owns the sphgpu context (created at the first calculation(), when the particle count is
// known).  A call uploads the particle vector (one bulk copy of the SPHParticle records),
// rebuilds the device octree on those positions, runs the stage and writes back only the members
// the reference module writes; the host tree Simulation::make_tree builds is not used.  Errors
// become THROW_ERROR (include/exception.hpp:9-14) with the library's message.
//
// Plug point, the module switch of Solver::initialize (src/solver.cpp:359-370):
//     auto gpu = std::make_shared<sph::gpu::Device>(SPHGPU_FP32_PAIR);
//     m_pre    = std::make_shared<sph::gpu::PreInteraction>(gpu);
//     m_fforce = std::make_shared<sph::gpu::FluidForce>(gpu);
//     m_gforce = std::make_shared<sph::gpu::GravityForce>(gpu);
#pragma once

#include <memory>

#include "defines.hpp"
#include "module.hpp"
#include "parameters.hpp"
#include "simulation.hpp"

#include "sphgpu.h"

namespace sph
{
namespace gpu
{

// sphgpu_params from the reference's parameter struct (include/parameters.hpp:20-79).
sphgpu_params to_c(const SPHParameters& p);

// Byte offsets of the SPHParticle members (include/particle.hpp:8-33).
sphgpu_aos_layout particle_layout();

class Device {
public:
    explicit Device(int precision = SPHGPU_FP32_PAIR) : m_precision(precision) {}
    ~Device();
    Device(const Device&) = delete;
    Device& operator=(const Device&) = delete;

    // Creates the context on the first call (n particles, the parameters of `param`).
    void attach(const SPHParameters& param, int n);
    // Whole SPHParticle records to the device (positions in the caller's order; the device
    // octree is rebuilt on them), simulation dt, and the gsph gradient arrays when `grads`.
    void upload(Simulation& sim, bool grads);
    // The members of `layout` (those >= 0) back into the records.
    void download(Simulation& sim, const sphgpu_aos_layout& layout);
    void download_grads(Simulation& sim);
    void check(int status, const char* what) const;
    sphgpu_ctx* context() const { return m_ctx; }
    int precision() const { return m_precision; }

private:
    sphgpu_ctx* m_ctx = nullptr;
    int m_precision;
    int m_n = 0;
    bool m_gsph = false;
};

class PreInteraction : public Module {
public:
    explicit PreInteraction(std::shared_ptr<Device> device) : m_device(std::move(device)) {}
    void initialize(std::shared_ptr<SPHParameters> param) override { m_param = param; }
    void calculation(std::shared_ptr<Simulation> sim) override;

private:
    std::shared_ptr<Device> m_device;
    std::shared_ptr<SPHParameters> m_param;
};

class FluidForce : public Module {
public:
    explicit FluidForce(std::shared_ptr<Device> device) : m_device(std::move(device)) {}
    void initialize(std::shared_ptr<SPHParameters> param) override { m_param = param; }
    void calculation(std::shared_ptr<Simulation> sim) override;

private:
    std::shared_ptr<Device> m_device;
    std::shared_ptr<SPHParameters> m_param;
};

class GravityForce : public Module {
public:
    explicit GravityForce(std::shared_ptr<Device> device) : m_device(std::move(device)) {}
    void initialize(std::shared_ptr<SPHParameters> param) override { m_param = param; }
    void calculation(std::shared_ptr<Simulation> sim) override;

private:
    std::shared_ptr<Device> m_device;
    std::shared_ptr<SPHParameters> m_param;
};

}  // namespace gpu
}  // namespace sph
