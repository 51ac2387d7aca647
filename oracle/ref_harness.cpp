// extern "C" harness around the reference SPH core, compiled together with the
// reference's own translation units (src/particle.cpp, src/kernels.cpp,
// src/spatial_hash.cpp, src/sph_engine.cpp) into oracle/_ref/libsph_ref.so by
// oracle/build_ref.sh.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links or loads this library; tests,
// the golden-fixture generator and the oracle validation use it to run the reference's
// own code on shared inputs.  Every function here only marshals flat float arrays into
// the reference's public types and calls the reference's public API:
//   * SpatialHash::build / query_squared          (src/spatial_hash.cpp:15-57)
//   * equations::compute_density / _pressure /
//     _pressure_force / _viscosity_force /
//     compute_external_forces / compute_acceleration (src/sph_engine.cpp:370-443)
//   * SPHEngine public methods                      (src/sph_engine.h:91-140)
//
// Parameter blocks are 16 floats in SPHParameters field order (src/sph_engine.h:14-34):
//   rest_density, gas_constant, viscosity, smoothing_length, particle_mass, timestep,
//   gravity, damping, CFL_factor, xmin, xmax, ymin, ymax, zmin, zmax,
//   neighbor_search_radius
#include <cstdint>
#include <cstring>
#include <vector>

#include "sph_engine.h"

namespace {

sph::SPHParameters unpack_params(const float* p) {
    sph::SPHParameters s;
    s.rest_density = p[0];
    s.gas_constant = p[1];
    s.viscosity = p[2];
    s.smoothing_length = p[3];
    s.particle_mass = p[4];
    s.timestep = p[5];
    s.gravity = p[6];
    s.damping = p[7];
    s.CFL_factor = p[8];
    s.bounds.xmin = p[9];
    s.bounds.xmax = p[10];
    s.bounds.ymin = p[11];
    s.bounds.ymax = p[12];
    s.bounds.zmin = p[13];
    s.bounds.zmax = p[14];
    s.neighbor_search_radius = p[15];
    return s;
}

void pack_params(const sph::SPHParameters& s, float* p) {
    p[0] = s.rest_density;
    p[1] = s.gas_constant;
    p[2] = s.viscosity;
    p[3] = s.smoothing_length;
    p[4] = s.particle_mass;
    p[5] = s.timestep;
    p[6] = s.gravity;
    p[7] = s.damping;
    p[8] = s.CFL_factor;
    p[9] = s.bounds.xmin;
    p[10] = s.bounds.xmax;
    p[11] = s.bounds.ymin;
    p[12] = s.bounds.ymax;
    p[13] = s.bounds.zmin;
    p[14] = s.bounds.zmax;
    p[15] = s.neighbor_search_radius;
}

std::vector<glm::vec3> to_vec3(size_t n, const float* a) {
    std::vector<glm::vec3> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = glm::vec3(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return v;
}

std::vector<sph::Particle> make_particles(size_t n, const float* pos, const float* vel,
                                          const float* mass) {
    std::vector<sph::Particle> ps;
    ps.reserve(n);
    for (size_t i = 0; i < n; ++i) {
        sph::Particle p(glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), mass[i],
                        sph::ParticleType::FLUID);
        if (vel) p.velocity = glm::vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        ps.push_back(p);
    }
    return ps;
}

}  // namespace

extern "C" {

// Neighbour lists exactly as SPHEngine::update_neighbor_lists builds them
// (src/sph_engine.cpp:335-353): SpatialHash with cell size = search radius, one
// query_squared per particle with radius^2 = r*r.  counts[i] receives |N(i)|; when idx is
// non-null it receives the concatenated lists in the reference's own order.  Returns the
// total number of pairs.
int64_t ref_query(size_t n, const float* pos, float cell_size, float radius,
                  int64_t* counts, int64_t* idx) {
    sph::SpatialHash hash(cell_size);
    hash.set_cell_size(cell_size);
    std::vector<glm::vec3> p = to_vec3(n, pos);
    hash.build(p);
    const float r2 = radius * radius;
    int64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        std::vector<size_t> nb = hash.query_squared(p[i], r2);
        counts[i] = static_cast<int64_t>(nb.size());
        if (idx)
            for (size_t k = 0; k < nb.size(); ++k) idx[total + k] = static_cast<int64_t>(nb[k]);
        total += static_cast<int64_t>(nb.size());
    }
    return total;
}

// One evaluation of the step's field phases on a given state, through the reference's
// own equations:: functions and the kernel create_kernel(kind, h) returns (kind 0
// CUBIC_SPLINE -- the engine's own choice --, 1 WENDLAND_C2, 2 GAUSSIAN; kernels.h:94-98)
// (the loop bodies of compute_densities / compute_pressures / compute_forces,
// src/sph_engine.cpp:203-244).  Writes rho[n], P[n], acc[3n].
void ref_fields_k(int kind, size_t n, const float* pos, const float* vel, const float* mass,
                  const float* params16, float* rho, float* P, float* acc) {
    const sph::SPHParameters prm = unpack_params(params16);
    sph::ParticleSystem ps(n > 0 ? n : 1);
    ps.add_particles(make_particles(n, pos, vel, mass));
    auto kernel = sph::create_kernel(static_cast<sph::KernelType>(kind), prm.smoothing_length);
    sph::SpatialHash hash(prm.smoothing_length);
    hash.set_cell_size(prm.neighbor_search_radius);
    std::vector<glm::vec3> p = ps.get_positions();
    hash.build(p);
    std::vector<std::vector<size_t>> nl(n);
    const float r2 = prm.neighbor_search_radius * prm.neighbor_search_radius;
#pragma omp parallel for
    for (size_t i = 0; i < n; ++i) nl[i] = hash.query_squared(ps[i].position, r2);
    std::vector<float> dens(n), pres(n);
#pragma omp parallel for
    for (size_t i = 0; i < n; ++i) dens[i] = sph::equations::compute_density(i, nl[i], ps, *kernel);
    for (size_t i = 0; i < n; ++i)
        pres[i] = sph::equations::compute_pressure(dens[i], prm.rest_density, prm.gas_constant);
#pragma omp parallel for
    for (size_t i = 0; i < n; ++i) {
        glm::vec3 fp = sph::equations::compute_pressure_force(i, nl[i], ps, *kernel, pres, dens);
        glm::vec3 fv =
            sph::equations::compute_viscosity_force(i, nl[i], ps, *kernel, prm.viscosity, dens);
        glm::vec3 fe = sph::equations::compute_external_forces(prm.gravity);
        glm::vec3 a = sph::equations::compute_acceleration(fp, fv, fe, ps[i].mass);
        acc[3 * i] = a.x;
        acc[3 * i + 1] = a.y;
        acc[3 * i + 2] = a.z;
    }
    for (size_t i = 0; i < n; ++i) {
        rho[i] = dens[i];
        P[i] = pres[i];
    }
}

void ref_fields(size_t n, const float* pos, const float* vel, const float* mass,
                const float* params16, float* rho, float* P, float* acc) {
    ref_fields_k(0, n, pos, vel, mass, params16, rho, P, acc);
}

// W, gradW and laplacianW of create_kernel(kind, h) at n vectors r[3n]
// (src/kernels.cpp:140-153, 172-200, 210-225).
void ref_kernel_eval(int kind, float h, size_t n, const float* r, float* w, float* grad,
                     float* lap) {
    auto kernel = sph::create_kernel(static_cast<sph::KernelType>(kind), h);
    for (size_t i = 0; i < n; ++i) {
        const glm::vec3 v(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
        w[i] = kernel->W(v);
        const glm::vec3 g = kernel->gradW(v);
        grad[3 * i] = g.x;
        grad[3 * i + 1] = g.y;
        grad[3 * i + 2] = g.z;
        lap[i] = kernel->laplacianW(v);
    }
}

// ---- SPHEngine handle API: drives the reference engine itself -------------------------
void* ref_engine_new(size_t capacity) { return new sph::SPHEngine(capacity); }
void ref_engine_free(void* e) { delete static_cast<sph::SPHEngine*>(e); }
void ref_engine_initialize(void* e, const float* p16) {
    static_cast<sph::SPHEngine*>(e)->initialize(unpack_params(p16));
}
void ref_engine_set_parameters(void* e, const float* p16) {
    static_cast<sph::SPHEngine*>(e)->set_parameters(unpack_params(p16));
}
void ref_engine_get_parameters(void* e, float* p16) {
    pack_params(static_cast<sph::SPHEngine*>(e)->get_parameters(), p16);
}
void ref_engine_set_smoothing_length(void* e, float h) {
    static_cast<sph::SPHEngine*>(e)->set_smoothing_length(h);
}
void ref_engine_set_gravity(void* e, float g) { static_cast<sph::SPHEngine*>(e)->set_gravity(g); }
void ref_engine_set_viscosity(void* e, float v) {
    static_cast<sph::SPHEngine*>(e)->set_viscosity(v);
}
void ref_engine_set_boundaries(void* e, const float* b6) {
    static_cast<sph::SPHEngine*>(e)->set_boundaries(b6[0], b6[1], b6[2], b6[3], b6[4], b6[5]);
}
void ref_engine_add(void* e, size_t n, const float* pos, const float* vel, const float* mass) {
    static_cast<sph::SPHEngine*>(e)->add_particles(make_particles(n, pos, vel, mass));
}
void ref_engine_clear(void* e) { static_cast<sph::SPHEngine*>(e)->clear_particles(); }
void ref_engine_init_scene(void* e, int which) {
    auto* eng = static_cast<sph::SPHEngine*>(e);
    if (which == 0) eng->initialize_dam_break();
    else if (which == 1) eng->initialize_fluid_drop();
    else eng->initialize_granular_flow();
}
void ref_engine_step(void* e, float dt) { static_cast<sph::SPHEngine*>(e)->step(dt); }
void ref_engine_run_steps(void* e, size_t k, int adaptive) {
    static_cast<sph::SPHEngine*>(e)->run_steps(k, adaptive != 0);
}
size_t ref_engine_size(void* e) { return static_cast<sph::SPHEngine*>(e)->get_particles().size(); }
size_t ref_engine_capacity(void* e) {
    return static_cast<sph::SPHEngine*>(e)->get_particles().capacity();
}
float ref_engine_time(void* e) { return static_cast<sph::SPHEngine*>(e)->get_current_time(); }
size_t ref_engine_step_count(void* e) { return static_cast<sph::SPHEngine*>(e)->get_step_count(); }
int ref_engine_initialized(void* e) { return static_cast<sph::SPHEngine*>(e)->is_initialized(); }

// pos/vel: 3*size floats in insertion order; rho/P: get_densities()/get_pressures(),
// which are capacity-length (src/sph_engine.h:135-136 with src/sph_engine.cpp:26-27).
// Returns the length of the density vector.
size_t ref_engine_get(void* e, float* pos, float* vel, float* rho, float* P) {
    auto* eng = static_cast<sph::SPHEngine*>(e);
    std::vector<glm::vec3> x = eng->get_positions(), v = eng->get_velocities();
    for (size_t i = 0; i < x.size(); ++i) {
        if (pos) { pos[3 * i] = x[i].x; pos[3 * i + 1] = x[i].y; pos[3 * i + 2] = x[i].z; }
        if (vel) { vel[3 * i] = v[i].x; vel[3 * i + 1] = v[i].y; vel[3 * i + 2] = v[i].z; }
    }
    std::vector<float> d = eng->get_densities(), p = eng->get_pressures();
    if (rho) std::memcpy(rho, d.data(), d.size() * sizeof(float));
    if (P) std::memcpy(P, p.data(), p.size() * sizeof(float));
    return d.size();
}

// Per-particle record fields of get_particles() (src/particle.h:17-49), 19 floats each:
// pos3 vel3 acc3 density pressure mass type temperature viscosity id color3
void ref_engine_particles(void* e, float* out) {
    const auto& ps = static_cast<sph::SPHEngine*>(e)->get_particles();
    for (size_t i = 0; i < ps.size(); ++i) {
        const sph::Particle& p = ps[i];
        float* o = out + 19 * i;
        o[0] = p.position.x; o[1] = p.position.y; o[2] = p.position.z;
        o[3] = p.velocity.x; o[4] = p.velocity.y; o[5] = p.velocity.z;
        o[6] = p.acceleration.x; o[7] = p.acceleration.y; o[8] = p.acceleration.z;
        o[9] = p.density; o[10] = p.pressure; o[11] = p.mass;
        o[12] = static_cast<float>(static_cast<int>(p.type));
        o[13] = p.temperature; o[14] = p.viscosity; o[15] = static_cast<float>(p.id);
        o[16] = p.color.x; o[17] = p.color.y; o[18] = p.color.z;
    }
}

// total_mass, total_energy, mass_error, energy_error, max_neighbors,
// total_neighbor_queries (src/sph_engine.cpp:178-200, src/sph_engine.h:51-59)
void ref_engine_diag(void* e, double* out6) {
    auto* eng = static_cast<sph::SPHEngine*>(e);
    float me = 0.0f, ee = 0.0f;
    eng->compute_conservation_errors(me, ee);
    out6[0] = eng->get_total_mass();
    out6[1] = eng->get_total_energy();
    out6[2] = me;
    out6[3] = ee;
    const auto& st = eng->get_performance_stats();
    out6[4] = static_cast<double>(st.max_neighbors);
    out6[5] = static_cast<double>(st.total_neighbor_queries);
}

}  // extern "C"
