// GPU drop-ins for the reference's PreInteraction, FluidForce and GravityForce modules over the
// sphgpu C-ABI.  See gpu_modules.hpp for the contract.
#include "gpu_modules.hpp"

#include <cstddef>
#include <string>
#include <vector>

#include "exception.hpp"
#include "particle.hpp"

namespace sph
{
namespace gpu
{

sphgpu_params to_c(const SPHParameters& p)
{
    sphgpu_params c{};
    c.sph_type = p.type == SPHType::SSPH ? 0 : p.type == SPHType::DISPH ? 1 : 2;
    c.kernel = p.kernel == KernelType::CUBIC_SPLINE ? 0 : 1;
    c.cfl_sound = p.cfl.sound;
    c.cfl_force = p.cfl.force;
    c.av_alpha = p.av.alpha;
    c.use_balsara = p.av.use_balsara_switch ? 1 : 0;
    c.use_tdav = p.av.use_time_dependent_av ? 1 : 0;
    c.alpha_max = p.av.alpha_max;
    c.alpha_min = p.av.alpha_min;
    c.epsilon_av = p.av.epsilon;
    c.use_ac = p.ac.is_valid ? 1 : 0;
    c.alpha_ac = p.ac.alpha;
    c.max_level = p.tree.max_level;
    c.leaf_num = p.tree.leaf_particle_num;
    c.neighbor_number = p.physics.neighbor_number;
    c.gamma = p.physics.gamma;
    c.iterative_sml = p.iterative_sml ? 1 : 0;
    c.periodic = p.periodic.is_valid ? 1 : 0;
    for (int k = 0; k < DIM; ++k) {
        c.range_min[k] = p.periodic.range_min[k];
        c.range_max[k] = p.periodic.range_max[k];
    }
    c.use_gravity = p.gravity.is_valid ? 1 : 0;
    c.g_constant = p.gravity.constant;
    c.theta = p.gravity.theta;
    c.gsph_2nd_order = p.gsph.is_2nd_order ? 1 : 0;
    return c;
}

sphgpu_aos_layout particle_layout()
{
    sphgpu_aos_layout l{};
    l.stride = sizeof(SPHParticle);
    l.pos = offsetof(SPHParticle, pos);
    l.vel = offsetof(SPHParticle, vel);
    l.vel_p = offsetof(SPHParticle, vel_p);
    l.acc = offsetof(SPHParticle, acc);
    l.mass = offsetof(SPHParticle, mass);
    l.dens = offsetof(SPHParticle, dens);
    l.pres = offsetof(SPHParticle, pres);
    l.ene = offsetof(SPHParticle, ene);
    l.ene_p = offsetof(SPHParticle, ene_p);
    l.dene = offsetof(SPHParticle, dene);
    l.sml = offsetof(SPHParticle, sml);
    l.sound = offsetof(SPHParticle, sound);
    l.balsara = offsetof(SPHParticle, balsara);
    l.alpha = offsetof(SPHParticle, alpha);
    l.gradh = offsetof(SPHParticle, gradh);
    l.phi = offsetof(SPHParticle, phi);
    l.neighbor = offsetof(SPHParticle, neighbor);
    return l;
}

namespace
{

// A layout naming only the given members (the others -1: not written back).
sphgpu_aos_layout only(std::initializer_list<long sphgpu_aos_layout::*> members)
{
    const sphgpu_aos_layout all = particle_layout();
    sphgpu_aos_layout l{};
    l.stride = all.stride;
    for (long sphgpu_aos_layout::*m : {&sphgpu_aos_layout::pos, &sphgpu_aos_layout::vel,
                                       &sphgpu_aos_layout::vel_p, &sphgpu_aos_layout::acc,
                                       &sphgpu_aos_layout::mass, &sphgpu_aos_layout::dens,
                                       &sphgpu_aos_layout::pres, &sphgpu_aos_layout::ene,
                                       &sphgpu_aos_layout::ene_p, &sphgpu_aos_layout::dene,
                                       &sphgpu_aos_layout::sml, &sphgpu_aos_layout::sound,
                                       &sphgpu_aos_layout::balsara, &sphgpu_aos_layout::alpha,
                                       &sphgpu_aos_layout::gradh, &sphgpu_aos_layout::phi,
                                       &sphgpu_aos_layout::neighbor})
        l.*m = -1;
    for (long sphgpu_aos_layout::*m : members) l.*m = all.*m;
    return l;
}

// Names of the gsph gradient arrays (src/solver.cpp:373-385) and their sphgpu fields.
const char* const GRAD_NAMES[3] = {"grad_velocity_0", "grad_velocity_1", "grad_velocity_2"};

}  // namespace

Device::~Device()
{
    if (m_ctx) sphgpu_destroy(m_ctx);
}

void Device::check(int status, const char* what) const
{
    if (status != SPHGPU_OK) THROW_ERROR("sphgpu ", what, ": ", sphgpu_last_error(m_ctx));
}

void Device::attach(const SPHParameters& param, int n)
{
    if (m_ctx) {
        if (n != m_n) THROW_ERROR("sphgpu: the particle number changed from ", m_n, " to ", n);
        return;
    }
    const sphgpu_params c = to_c(param);
    sphgpu_ctx* ctx = nullptr;
    const int rc = sphgpu_create(&c, DIM, n, m_precision, &ctx);
    if (rc != SPHGPU_OK) THROW_ERROR("sphgpu create: ", sphgpu_last_error(nullptr));
    // the modules are driven one stage at a time by the Solver: the schedule tuner of the
    // whole-step entry points does not run
    sphgpu_set_tuning(ctx, 4, 0);
    m_ctx = ctx;
    m_n = n;
    m_gsph = param.type == SPHType::GSPH;
}

void Device::upload(Simulation& sim, bool grads)
{
    const sphgpu_aos_layout l = particle_layout();
    check(sphgpu_upload_aos(m_ctx, sim.get_particles().data(), &l), "upload");
    check(sphgpu_set_scalar(m_ctx, SPHGPU_DT, 0, sim.get_dt()), "set dt");
    if (grads && m_gsph) {
        // grad rho, grad P and the rows of grad v, gathered into the field layouts of the ABI
        const int n = m_n;
        std::vector<double> buf((size_t)n * DIM * DIM);
        auto put_vec = [&](const char* name, int field) {
            const auto& a = sim.get_vector_array(name);
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < DIM; ++k) buf[(size_t)i * DIM + k] = a[i][k];
            check(sphgpu_set_field(m_ctx, field, buf.data()), "set gradient");
        };
        put_vec("grad_density", SPHGPU_GRAD_D);
        put_vec("grad_pressure", SPHGPU_GRAD_P);
        for (int a = 0; a < DIM; ++a) {
            const auto& g = sim.get_vector_array(GRAD_NAMES[a]);
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < DIM; ++k) buf[((size_t)i * DIM + a) * DIM + k] = g[i][k];
        }
        check(sphgpu_set_field(m_ctx, SPHGPU_GRAD_V, buf.data()), "set gradient");
    }
    check(sphgpu_make_tree(m_ctx), "make_tree");
}

void Device::download(Simulation& sim, const sphgpu_aos_layout& layout)
{
    check(sphgpu_download_aos(m_ctx, sim.get_particles().data(), &layout), "download");
}

void Device::download_grads(Simulation& sim)
{
    const int n = m_n;
    std::vector<double> buf((size_t)n * DIM * DIM);
    auto get_vec = [&](const char* name, int field) {
        check(sphgpu_get_field(m_ctx, field, buf.data()), "get gradient");
        auto& a = sim.get_vector_array(name);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < DIM; ++k) a[i][k] = buf[(size_t)i * DIM + k];
    };
    get_vec("grad_density", SPHGPU_GRAD_D);
    get_vec("grad_pressure", SPHGPU_GRAD_P);
    check(sphgpu_get_field(m_ctx, SPHGPU_GRAD_V, buf.data()), "get gradient");
    for (int a = 0; a < DIM; ++a) {
        auto& g = sim.get_vector_array(GRAD_NAMES[a]);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < DIM; ++k) g[i][k] = buf[((size_t)i * DIM + a) * DIM + k];
    }
}

void PreInteraction::calculation(std::shared_ptr<Simulation> sim)
{
    Device& d = *m_device;
    d.attach(*m_param, sim->get_particle_num());
    d.upload(*sim, false);
    d.check(sphgpu_pre_interaction(d.context()), "pre_interaction");
    double hv = 0.0;
    d.check(sphgpu_get_scalar(d.context(), SPHGPU_H_PER_V_SIG, 0, &hv), "h_per_v_sig");
    // the members PreInteraction writes (the first call's initial_smoothing included)
    d.download(*sim, only({&sphgpu_aos_layout::sml, &sphgpu_aos_layout::dens, &sphgpu_aos_layout::pres,
                           &sphgpu_aos_layout::gradh, &sphgpu_aos_layout::balsara,
                           &sphgpu_aos_layout::alpha, &sphgpu_aos_layout::neighbor}));
    if (m_param->type == SPHType::GSPH) d.download_grads(*sim);
    sim->set_h_per_v_sig(hv);
}

void FluidForce::calculation(std::shared_ptr<Simulation> sim)
{
    Device& d = *m_device;
    d.attach(*m_param, sim->get_particle_num());
    d.upload(*sim, true);
    d.check(sphgpu_fluid_force(d.context()), "fluid_force");
    d.download(*sim, only({&sphgpu_aos_layout::acc, &sphgpu_aos_layout::dene}));
}

void GravityForce::calculation(std::shared_ptr<Simulation> sim)
{
    if (!m_param->gravity.is_valid) return;   // src/gravity_force.cpp:54-56
    Device& d = *m_device;
    d.attach(*m_param, sim->get_particle_num());
    d.upload(*sim, false);
    d.check(sphgpu_gravity_force(d.context()), "gravity_force");
    d.download(*sim, only({&sphgpu_aos_layout::acc, &sphgpu_aos_layout::phi}));
}

}  // namespace gpu
}  // namespace sph
