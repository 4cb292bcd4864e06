/*
 * Driver around the reference's own hot-path translation units — TEST INFRASTRUCTURE ONLY.
 *
 * Built by oracle/build_ref.sh against the reference's headers (with DIM set per build) and
 * linked with the reference's unmodified src/{simulation,bhtree,exhaustive_search,
 * pre_interaction,fluid_force,gravity_force,timestep}.cpp, src/disph/*.cpp, src/gsph/*.cpp.
 * The reference's Solver, Output and Logger sources need Boost, which is absent, so this file
 * restates the few lines of glue around the modules:
 *   - SPHParameters are filled from the C struct orc_params (keys of src/solver.cpp:193-298);
 *   - the Logger statics of src/logger.cpp:17-19 are defined here (log stream left closed);
 *   - Solver::initialize (src/solver.cpp:353-415), Solver::integrate (:417-429),
 *     Solver::predict (:431-456) and Solver::correct (:458-474) are restated below.
 * Exported symbols use the prefix refD_ with the same signatures as the orcD_ functions of
 * oracle/sph_oracle.h.
 */
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>
#include <string>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "defines.hpp"
#include "parameters.hpp"
#include "particle.hpp"
#include "simulation.hpp"
#include "periodic.hpp"
#include "bhtree.hpp"
#include "exception.hpp"
#include "logger.hpp"
#include "exhaustive_search.hpp"
#include "timestep.hpp"
#include "pre_interaction.hpp"
#include "fluid_force.hpp"
#include "gravity_force.hpp"
#include "disph/d_pre_interaction.hpp"
#include "disph/d_fluid_force.hpp"
#include "gsph/g_pre_interaction.hpp"
#include "gsph/g_fluid_force.hpp"

#include "sph_oracle.h"

#ifdef USE_SPHGPU
// The GPU Module drop-ins (sphcode_gb300/cxx/gpu_modules.hpp) in place of the reference's
// PreInteraction, FluidForce and GravityForce: the plug point of Solver::initialize
// (src/solver.cpp:359-370), the rest of the Solver glue unchanged.
#include "gpu_modules.hpp"
static int g_gpu_precision = SPHGPU_FP64;
#endif

namespace sph {
std::string Logger::dir_name;
std::ofstream Logger::log_io;
bool Logger::open_flag = false;
}

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define API(name) CAT(CAT(ref, DIM), CAT(_, name))

namespace {

struct Ref {
    std::shared_ptr<sph::SPHParameters> param;
    std::shared_ptr<sph::Simulation> sim;
    std::shared_ptr<sph::Module> timestep, pre, fforce, gforce;
    bool tree_sized = false;
};

std::shared_ptr<sph::SPHParameters> make_params(const orc_params* p)
{
    auto q = std::make_shared<sph::SPHParameters>();
    q->time.start = 0.0;
    q->time.end = 1.0;
    q->time.output = 1.0;
    q->time.energy = 1.0;
    q->type = p->sph_type == 0 ? sph::SPHType::SSPH : p->sph_type == 1 ? sph::SPHType::DISPH : sph::SPHType::GSPH;
    q->cfl.sound = p->cfl_sound;
    q->cfl.force = p->cfl_force;
    q->av.alpha = p->av_alpha;
    q->av.use_balsara_switch = p->use_balsara != 0;
    q->av.use_time_dependent_av = p->use_tdav != 0;
    q->av.alpha_max = p->alpha_max;
    q->av.alpha_min = p->alpha_min;
    q->av.epsilon = p->epsilon_av;
    q->ac.is_valid = p->use_ac != 0;
    q->ac.alpha = p->alpha_ac;
    q->tree.max_level = p->max_level;
    q->tree.leaf_particle_num = p->leaf_num;
    q->physics.neighbor_number = p->neighbor_number;
    q->physics.gamma = p->gamma;
    q->kernel = p->kernel == 0 ? sph::KernelType::CUBIC_SPLINE : sph::KernelType::WENDLAND;
    q->iterative_sml = p->iterative_sml != 0;
    q->periodic.is_valid = p->periodic != 0;
    for (int k = 0; k < DIM; ++k) {
        q->periodic.range_min[k] = p->range_min[k];
        q->periodic.range_max[k] = p->range_max[k];
    }
    q->gravity.is_valid = p->use_gravity != 0;
    q->gravity.constant = p->g_constant;
    q->gravity.theta = p->theta;
    q->gsph.is_2nd_order = p->gsph_2nd_order != 0;
    return q;
}

void predict(Ref* r)
{
    auto& p = r->sim->get_particles();
    const int num = r->sim->get_particle_num();
    auto* periodic = r->sim->get_periodic().get();
    const real dt = r->sim->get_dt();
    const real gamma = r->param->physics.gamma;
    const real c_sound = gamma * (gamma - 1.0);
#pragma omp parallel for
    for (int i = 0; i < num; ++i) {
        p[i].vel_p = p[i].vel + p[i].acc * (0.5 * dt);
        p[i].ene_p = p[i].ene + p[i].dene * (0.5 * dt);
        p[i].pos += p[i].vel_p * dt;
        p[i].vel += p[i].acc * dt;
        p[i].ene += p[i].dene * dt;
        p[i].sound = std::sqrt(c_sound * p[i].ene);
        periodic->apply(p[i].pos);
    }
}

void correct(Ref* r)
{
    auto& p = r->sim->get_particles();
    const int num = r->sim->get_particle_num();
    const real dt = r->sim->get_dt();
    const real gamma = r->param->physics.gamma;
    const real c_sound = gamma * (gamma - 1.0);
#pragma omp parallel for
    for (int i = 0; i < num; ++i) {
        p[i].vel = p[i].vel_p + p[i].acc * (0.5 * dt);
        p[i].ene = p[i].ene_p + p[i].dene * (0.5 * dt);
        p[i].sound = std::sqrt(c_sound * p[i].ene);
    }
}

void init_fields(Ref* r)
{
    auto& p = r->sim->get_particles();
    const int num = r->sim->get_particle_num();
    const real gamma = r->param->physics.gamma;
    const real c_sound = gamma * (gamma - 1.0);
    const real alpha = r->param->av.alpha;
    for (int i = 0; i < num; ++i) {
        p[i].alpha = alpha;
        p[i].balsara = 1.0;
        p[i].sound = std::sqrt(c_sound * p[i].ene);
    }
}

void make_tree(Ref* r)
{
    if (!r->tree_sized) {
        r->sim->get_tree()->resize(r->sim->get_particle_num());
        r->tree_sized = true;
    }
    r->sim->make_tree();
}

std::string g_last_exception;

template <typename F>
int guarded(F&& f)
{
    try {
        f();
    } catch (std::exception& e) {
        g_last_exception = e.what();
        return ORC_ERR_EXCEPTION;
    }
    return 0;
}

std::vector<vec_t>* grad_array(Ref* r, const char* name)
{
    if (r->param->type != sph::SPHType::GSPH) return nullptr;
    return &r->sim->get_vector_array(name);
}

}  // namespace

extern "C" {

void* API(create)(const orc_params* p, int n)
{
    if (!p || n <= 0) return nullptr;
    auto* r = new Ref();
    r->param = make_params(p);
    r->sim = std::make_shared<sph::Simulation>(r->param);
    std::vector<sph::SPHParticle> parts(n);
    for (int i = 0; i < n; ++i) parts[i].id = i;
    r->sim->set_particles(parts);
    r->sim->set_particle_num(n);
    r->timestep = std::make_shared<sph::TimeStep>();
    if (r->param->type == sph::SPHType::SSPH) {
        r->pre = std::make_shared<sph::PreInteraction>();
        r->fforce = std::make_shared<sph::FluidForce>();
    } else if (r->param->type == sph::SPHType::DISPH) {
        r->pre = std::make_shared<sph::disph::PreInteraction>();
        r->fforce = std::make_shared<sph::disph::FluidForce>();
    } else {
        r->pre = std::make_shared<sph::gsph::PreInteraction>();
        r->fforce = std::make_shared<sph::gsph::FluidForce>();
        std::vector<std::string> names = {"grad_density", "grad_pressure", "grad_velocity_0"};
#if DIM >= 2
        names.push_back("grad_velocity_1");
#endif
#if DIM == 3
        names.push_back("grad_velocity_2");
#endif
        r->sim->add_vector_array(names);
    }
    r->gforce = std::make_shared<sph::GravityForce>();
#ifdef USE_SPHGPU
    {
        auto dev = std::make_shared<sph::gpu::Device>(g_gpu_precision);
        r->pre = std::make_shared<sph::gpu::PreInteraction>(dev);
        r->fforce = std::make_shared<sph::gpu::FluidForce>(dev);
        r->gforce = std::make_shared<sph::gpu::GravityForce>(dev);
    }
#endif
    r->timestep->initialize(r->param);
    r->pre->initialize(r->param);
    r->fforce->initialize(r->param);
    r->gforce->initialize(r->param);
    return r;
}

void API(destroy)(void* h) { delete static_cast<Ref*>(h); }

int API(set_field)(void* h, int f, const double* src)
{
    auto* r = static_cast<Ref*>(h);
    auto& p = r->sim->get_particles();
    const int n = r->sim->get_particle_num();
    for (int i = 0; i < n; ++i) {
        auto& q = p[i];
        switch (f) {
        case ORC_POS: for (int k = 0; k < DIM; ++k) q.pos[k] = src[i * DIM + k]; break;
        case ORC_VEL: for (int k = 0; k < DIM; ++k) q.vel[k] = src[i * DIM + k]; break;
        case ORC_VEL_P: for (int k = 0; k < DIM; ++k) q.vel_p[k] = src[i * DIM + k]; break;
        case ORC_ACC: for (int k = 0; k < DIM; ++k) q.acc[k] = src[i * DIM + k]; break;
        case ORC_MASS: q.mass = src[i]; break;
        case ORC_DENS: q.dens = src[i]; break;
        case ORC_PRES: q.pres = src[i]; break;
        case ORC_ENE: q.ene = src[i]; break;
        case ORC_ENE_P: q.ene_p = src[i]; break;
        case ORC_DENE: q.dene = src[i]; break;
        case ORC_SML: q.sml = src[i]; break;
        case ORC_SOUND: q.sound = src[i]; break;
        case ORC_BALSARA: q.balsara = src[i]; break;
        case ORC_ALPHA: q.alpha = src[i]; break;
        case ORC_GRADH: q.gradh = src[i]; break;
        case ORC_PHI: q.phi = src[i]; break;
        case ORC_NEIGHBOR: q.neighbor = (int)src[i]; break;
        case ORC_GRAD_D:
        case ORC_GRAD_P: {
            auto* g = grad_array(r, f == ORC_GRAD_D ? "grad_density" : "grad_pressure");
            if (!g) return ORC_ERR_ARG;
            for (int k = 0; k < DIM; ++k) (*g)[i][k] = src[i * DIM + k];
            break;
        }
        case ORC_GRAD_V: {
            for (int a = 0; a < DIM; ++a) {
                const std::string name = "grad_velocity_" + std::to_string(a);
                auto* g = grad_array(r, name.c_str());
                if (!g) return ORC_ERR_ARG;
                for (int k = 0; k < DIM; ++k) (*g)[i][k] = src[(i * DIM + a) * DIM + k];
            }
            break;
        }
        default: return ORC_ERR_ARG;
        }
    }
    return 0;
}

int API(get_field)(void* h, int f, double* dst)
{
    auto* r = static_cast<Ref*>(h);
    auto& p = r->sim->get_particles();
    const int n = r->sim->get_particle_num();
    for (int i = 0; i < n; ++i) {
        const auto& q = p[i];
        switch (f) {
        case ORC_POS: for (int k = 0; k < DIM; ++k) dst[i * DIM + k] = q.pos[k]; break;
        case ORC_VEL: for (int k = 0; k < DIM; ++k) dst[i * DIM + k] = q.vel[k]; break;
        case ORC_VEL_P: for (int k = 0; k < DIM; ++k) dst[i * DIM + k] = q.vel_p[k]; break;
        case ORC_ACC: for (int k = 0; k < DIM; ++k) dst[i * DIM + k] = q.acc[k]; break;
        case ORC_MASS: dst[i] = q.mass; break;
        case ORC_DENS: dst[i] = q.dens; break;
        case ORC_PRES: dst[i] = q.pres; break;
        case ORC_ENE: dst[i] = q.ene; break;
        case ORC_ENE_P: dst[i] = q.ene_p; break;
        case ORC_DENE: dst[i] = q.dene; break;
        case ORC_SML: dst[i] = q.sml; break;
        case ORC_SOUND: dst[i] = q.sound; break;
        case ORC_BALSARA: dst[i] = q.balsara; break;
        case ORC_ALPHA: dst[i] = q.alpha; break;
        case ORC_GRADH: dst[i] = q.gradh; break;
        case ORC_PHI: dst[i] = q.phi; break;
        case ORC_NEIGHBOR: dst[i] = q.neighbor; break;
        case ORC_GRAD_D:
        case ORC_GRAD_P: {
            auto* g = grad_array(r, f == ORC_GRAD_D ? "grad_density" : "grad_pressure");
            if (!g) return ORC_ERR_ARG;
            for (int k = 0; k < DIM; ++k) dst[i * DIM + k] = (*g)[i][k];
            break;
        }
        case ORC_GRAD_V: {
            for (int a = 0; a < DIM; ++a) {
                const std::string name = "grad_velocity_" + std::to_string(a);
                auto* g = grad_array(r, name.c_str());
                if (!g) return ORC_ERR_ARG;
                for (int k = 0; k < DIM; ++k) dst[(i * DIM + a) * DIM + k] = (*g)[i][k];
            }
            break;
        }
        default: return ORC_ERR_ARG;
        }
    }
    return 0;
}

void API(set_scalar)(void* h, int which, double v)
{
    auto* r = static_cast<Ref*>(h);
    if (which == ORC_TIME) r->sim->set_time(v);
    else if (which == ORC_DT) r->sim->set_dt(v);
    else if (which == ORC_H_PER_V_SIG) r->sim->set_h_per_v_sig(v);
}

double API(get_scalar)(void* h, int which)
{
    auto* r = static_cast<Ref*>(h);
    if (which == ORC_TIME) return r->sim->get_time();
    if (which == ORC_DT) return r->sim->get_dt();
    return r->sim->get_h_per_v_sig();
}

int API(stage)(void* h, int stage)
{
    auto* r = static_cast<Ref*>(h);
    return guarded([&] {
        switch (stage) {
        case ORC_STAGE_TIMESTEP: r->timestep->calculation(r->sim); break;
        case ORC_STAGE_PREDICT: predict(r); break;
        case ORC_STAGE_MAKE_TREE: make_tree(r); break;
        case ORC_STAGE_PRE: r->pre->calculation(r->sim); break;
        case ORC_STAGE_FLUID: r->fforce->calculation(r->sim); break;
        case ORC_STAGE_GRAVITY: r->gforce->calculation(r->sim); break;
        case ORC_STAGE_CORRECT: correct(r); break;
        case ORC_STAGE_INIT_FIELDS: init_fields(r); break;
        }
    });
}

int API(initialize)(void* h)
{
    auto* r = static_cast<Ref*>(h);
    return guarded([&] {
        init_fields(r);
        make_tree(r);
        r->pre->calculation(r->sim);
        r->fforce->calculation(r->sim);
        r->gforce->calculation(r->sim);
    });
}

int API(step)(void* h)
{
    auto* r = static_cast<Ref*>(h);
    return guarded([&] {
        r->timestep->calculation(r->sim);
        predict(r);
        make_tree(r);
        r->pre->calculation(r->sim);
        r->fforce->calculation(r->sim);
        r->gforce->calculation(r->sim);
        correct(r);
        r->sim->update_time();
    });
}

int API(neighbors)(void* h, int is_ij, int exh, int* counts, int* list, int cap)
{
    auto* r = static_cast<Ref*>(h);
    auto& p = r->sim->get_particles();
    const int n = r->sim->get_particle_num();
    auto* tree = r->sim->get_tree().get();
    auto* periodic = r->sim->get_periodic().get();
#pragma omp parallel
    {
        std::vector<int> nl(cap);
#pragma omp for schedule(dynamic, 64)
        for (int i = 0; i < n; ++i) {
            const int nn = exh ? sph::exhaustive_search(p[i], p[i].sml, p, n, nl, cap, periodic, is_ij != 0)
                               : tree->neighbor_search(p[i], nl, p, is_ij != 0);
            counts[i] = nn;
            if (list)   // NULL: counts only
                for (int k = 0; k < nn && k < cap; ++k) list[(size_t)i * cap + k] = nl[k];
        }
    }
    return 0;
}

int API(tree_stats)(void* h, int* out)
{
    (void)h;
    std::memset(out, 0, sizeof(int) * 130);
    return ORC_ERR_ARG;   /* BHTree keeps its nodes private; shape is compared through the port */
}

void API(energy)(void* h, double* out)
{
    auto* r = static_cast<Ref*>(h);
    const auto& p = r->sim->get_particles();
    const int n = r->sim->get_particle_num();
    double ek = 0.0, et = 0.0, ep = 0.0, mom[DIM] = {0};
    for (int i = 0; i < n; ++i) {
        ek += 0.5 * p[i].mass * abs2(p[i].vel);
        et += p[i].mass * p[i].ene;
        ep += 0.5 * p[i].mass * p[i].phi;
        for (int k = 0; k < DIM; ++k) mom[k] += p[i].mass * p[i].vel[k];
    }
    out[0] = ek; out[1] = et; out[2] = ep; out[3] = ek + et + ep;
    for (int k = 0; k < DIM; ++k) out[4 + k] = mom[k];
}

int API(newton_failures)(void* h) { (void)h; return -1; }

// Text of the last exception a module threw (THROW_ERROR), for the caller's error message.
const char* API(last_exception)() { return g_last_exception.c_str(); }

#ifdef USE_SPHGPU
// Arithmetic form of the GPU modules of the contexts created from now on (sphgpu_precision).
void API(set_gpu_precision)(int precision) { g_gpu_precision = precision; }
#endif

void API(set_threads)(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // extern "C"
