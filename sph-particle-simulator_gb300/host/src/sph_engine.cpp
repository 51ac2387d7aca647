// GB300 drop-in SPHEngine: the reference's engine API (src/sph_engine.cpp) over the sphx
// C ABI.  Host code only marshals the particle set and parameters; every phase of step()
// runs on the GPU.  Built with -ffp-contract=off: the few host-side float formulas
// (get_total_mass, get_total_energy, scene generators) round exactly like the reference's.
#include "sph_engine.h"

#include <algorithm>
#include <cmath>
#include <iostream>
#include <stdexcept>
#include <string>

#include "sphx.h"

namespace sph {

namespace {

void check(int rc, const char* where) {
    if (rc != SPHX_OK)
        throw std::runtime_error(std::string(where) + ": " + sphx_strerror(rc));
}

sphx_params to_sphx(const SPHParameters& p) {
    sphx_params s;
    s.rest_density = p.rest_density;
    s.gas_constant = p.gas_constant;
    s.viscosity = p.viscosity;
    s.smoothing_length = p.smoothing_length;
    s.particle_mass = p.particle_mass;
    s.timestep = p.timestep;
    s.gravity = p.gravity;
    s.damping = p.damping;
    s.cfl_factor = p.CFL_factor;
    s.xmin = p.bounds.xmin;
    s.xmax = p.bounds.xmax;
    s.ymin = p.bounds.ymin;
    s.ymax = p.bounds.ymax;
    s.zmin = p.bounds.zmin;
    s.zmax = p.bounds.zmax;
    s.neighbor_search_radius = p.neighbor_search_radius;
    return s;
}

}  // namespace

SPHEngine::SPHEngine(size_t max_particles) : particles_(max_particles) {
    sphx_tuning t{};
    t.profile = 1;  // fill PerformanceStats' phase timers, like the reference
    check(sphx_create(&gpu_, max_particles > 0 ? max_particles : 1, &t), "sphx_create");
}

SPHEngine::~SPHEngine() {
    sphx_destroy(gpu_);
    sphx_free_host(stage_);
}

// Page-locked transfer buffers sized for the capacity C, made on first use, 15 floats per
// particle: the upload region x [0, 3C), v [3C, 6C), m [6C, 7C) -- read in place by the GPU
// when the stream reaches the upload, so written only after the stream went idle (every
// path that changes the host set downloads, and so synchronises, first) -- and the
// download region rho [7C, 8C), P [8C, 9C), x [9C, 12C), v [12C, 15C) for the single-field
// copies.  Null when page-locked memory is not available: the transfers then go through
// ordinary vectors.
//
// The upload region is kept equal to the mirror (`stage_current_`, first `staged_`
// particles): a download writes the device's x and v straight into it, an addition
// appends its particles, a clear empties it; step() then uploads it as it is.
float* SPHEngine::stage() const {
    if (!stage_) {
        void* p = nullptr;
        if (sphx_alloc_host(&p, 15 * sizeof(float) * std::max<size_t>(particles_.capacity(), 1)) ==
            SPHX_OK)
            stage_ = static_cast<float*>(p);
    }
    return stage_;
}

void SPHEngine::push_params() {
    const sphx_params p = to_sphx(params_);
    const int rc = sphx_set_params(gpu_, &p);
    // A non-positive search radius cannot define cells; the device keeps the last valid
    // parameters and step() reports the error.
    if (rc != SPHX_OK && rc != SPHX_ERR_INVALID_ARG) check(rc, "sphx_set_params");
}

// SPHEngine::initialize (src/sph_engine.cpp:20-33)
void SPHEngine::initialize(const SPHParameters& params) {
    params_ = params;
    push_params();
    densities_.resize(particles_.capacity());
    pressures_.resize(particles_.capacity());
    initialized_ = true;
    reset_performance_stats();
}

void SPHEngine::initialize_dam_break() {
    if (!initialized_) initialize(SPHParameters{});
    auto ps = utils::create_dam_break_setup(glm::vec3(0.4f, 0.6f, 0.8f),
                                            glm::vec3(0.2f, 0.4f, 0.8f), 0.01f, params_);
    replace_particles(ps);
}

void SPHEngine::initialize_fluid_drop() {
    if (!initialized_) initialize(SPHParameters{});
    auto ps = utils::create_fluid_drop_setup(glm::vec3(0.0f, 0.5f, 0.0f), 0.1f, 0.008f, params_);
    replace_particles(ps);
}

void SPHEngine::initialize_granular_flow() {
    if (!initialized_) initialize(SPHParameters{});
    auto ps = utils::create_granular_flow_setup(glm::vec3(0.3f, 0.4f, 0.8f),
                                                glm::vec3(1.0f, 1.0f, 1.0f), 0.012f, params_);
    replace_particles(ps);
}

// the initialize_* scenes: the host set replaced by `ps`
void SPHEngine::replace_particles(const std::vector<Particle>& ps) {
    host_will_change();
    particles_.clear();
    staged_ = 0;
    particles_.add_particles(ps);
    stage_append(0);
}

void SPHEngine::add_particles(const std::vector<Particle>& particles) {
    host_will_change();
    const size_t old = particles_.size();
    particles_.add_particles(particles);
    stage_append(old);
}

// SPHEngine::clear_particles (src/sph_engine.cpp:87-91)
void SPHEngine::clear_particles() {
    host_will_change();
    particles_.clear();
    staged_ = 0;
    step_count_ = 0;
    check(sphx_set_time(gpu_, 0.0f), "sphx_set_time");
}

// The mirror's particles [from, size()) appended to the upload region; the region stays
// current only if it held the first `from` of them.
void SPHEngine::stage_append(size_t from) {
    float* buf = stage();
    const size_t n = particles_.size();
    if (!buf || staged_ != from) {
        stage_current_ = false;
        return;
    }
    const size_t C = std::max<size_t>(particles_.capacity(), 1);
    float* x = buf;
    float* v = buf + 3 * C;
    float* m = buf + 6 * C;
    const long long a = static_cast<long long>(from), e = static_cast<long long>(n);
#pragma omp parallel for schedule(static) if (e - a > 65536)
    for (long long i = a; i < e; ++i) {
        const Particle& p = particles_[static_cast<size_t>(i)];
        x[3 * i] = p.position.x;
        x[3 * i + 1] = p.position.y;
        x[3 * i + 2] = p.position.z;
        v[3 * i] = p.velocity.x;
        v[3 * i + 1] = p.velocity.y;
        v[3 * i + 2] = p.velocity.z;
        m[i] = p.mass;
    }
    staged_ = n;
    stage_current_ = true;
}

void SPHEngine::host_will_change() {
    sync_to_host();
    device_dirty_ = true;
}

void SPHEngine::sync_to_device() {
    if (!device_dirty_) return;
    const size_t n = particles_.size();
    float* buf = stage();
    if (buf && !(stage_current_ && staged_ == n)) {  // rebuild the upload region
        staged_ = 0;
        stage_current_ = true;
        stage_append(0);
    }
    if (buf) {
        const size_t C = std::max<size_t>(particles_.capacity(), 1);
        check(sphx_upload(gpu_, n, buf, buf + 3 * C, buf + 6 * C), "sphx_upload");
        device_dirty_ = false;
        return;
    }
    std::vector<float> x(3 * std::max<size_t>(n, 1)), v(x.size()), m(std::max<size_t>(n, 1));
    const long long nn = static_cast<long long>(n);
#pragma omp parallel for schedule(static) if (nn > 65536)
    for (long long i = 0; i < nn; ++i) {
        const Particle& p = particles_[static_cast<size_t>(i)];
        x[3 * i] = p.position.x;
        x[3 * i + 1] = p.position.y;
        x[3 * i + 2] = p.position.z;
        v[3 * i] = p.velocity.x;
        v[3 * i + 1] = p.velocity.y;
        v[3 * i + 2] = p.velocity.z;
        m[i] = p.mass;
    }
    check(sphx_upload(gpu_, n, x.data(), v.data(), m.data()), "sphx_upload");
    device_dirty_ = false;
}

// Device -> host mirror: positions, velocities, densities and pressures of the last step
// (particle.density / particle.pressure are written like compute_densities /
// compute_pressures do, cpp:203-224; particle.acceleration is left as it is).  x and v
// arrive in the upload region, which then equals the mirror again.
void SPHEngine::sync_to_host() const {
    if (!host_stale_) return;
    const size_t n = particles_.size();
    const size_t C = std::max<size_t>(particles_.capacity(), 1);
    std::vector<float> fallback;
    float* buf = stage();
    float *x, *v, *rho, *P;
    if (buf) {
        x = buf;
        v = buf + 3 * C;
        rho = buf + 7 * C;
        P = buf + 8 * C;
    } else {
        fallback.resize(8 * std::max<size_t>(n, 1));
        x = fallback.data();
        v = x + 3 * n;
        rho = x + 6 * n;
        P = x + 7 * n;
    }
    check(sphx_download(gpu_, x, v, rho, P, nullptr), "sphx_download");
    const long long nn = static_cast<long long>(n);
    const size_t nd = densities_.size(), np = pressures_.size();
#pragma omp parallel for schedule(static) if (nn > 65536)
    for (long long i = 0; i < nn; ++i) {
        Particle& p = particles_[static_cast<size_t>(i)];
        p.position = glm::vec3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        p.velocity = glm::vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        p.density = rho[i];
        p.pressure = P[i];
        if (static_cast<size_t>(i) < nd) densities_[i] = rho[i];
        if (static_cast<size_t>(i) < np) pressures_[i] = P[i];
    }
    host_stale_ = false;
}

// One field of the current state into out (3 or 1 floats per particle), from the device
// when it holds a newer state than the mirror (the mirror is left as it is), else from the
// mirror.  field: 0 x, 1 v, 2 rho, 3 P.
void SPHEngine::copy_field(int field, float* out) const {
    const size_t n = particles_.size();
    if (n == 0) return;
    const long long nn = static_cast<long long>(n);
    const int w = field < 2 ? 3 : 1;
    if (!host_stale_) {
#pragma omp parallel for schedule(static) if (nn > 65536)
        for (long long i = 0; i < nn; ++i) {
            const Particle& p = particles_[static_cast<size_t>(i)];
            if (field == 0 || field == 1) {
                const glm::vec3& q = field == 0 ? p.position : p.velocity;
                out[3 * i] = q.x;
                out[3 * i + 1] = q.y;
                out[3 * i + 2] = q.z;
            } else {
                out[i] = field == 2 ? p.density : p.pressure;
            }
        }
        return;
    }
    float* buf = stage();
    const size_t C = std::max<size_t>(particles_.capacity(), 1);
    float* tmp = buf ? buf + (field == 0 ? 9 * C : field == 1 ? 12 * C : field == 2 ? 7 * C : 8 * C)
                     : out;
    check(sphx_download(gpu_, field == 0 ? tmp : nullptr, field == 1 ? tmp : nullptr,
                        field == 2 ? tmp : nullptr, field == 3 ? tmp : nullptr, nullptr),
          "sphx_download");
    if (tmp == out) return;
    const long long words = nn * w;
#pragma omp parallel for schedule(static) if (words > 65536)
    for (long long i = 0; i < words; ++i) out[i] = tmp[i];
}

void SPHEngine::copy_positions(float* out) const { copy_field(0, out); }
void SPHEngine::copy_velocities(float* out) const { copy_field(1, out); }

// densities / pressures: the capacity-length vectors get_densities / get_pressures return
void SPHEngine::copy_densities(float* out) const {
    const size_t n = std::min(particles_.size(), densities_.size());
    std::copy(densities_.begin() + static_cast<std::ptrdiff_t>(n), densities_.end(), out + n);
    if (n) copy_field(2, out);
}
void SPHEngine::copy_pressures(float* out) const {
    const size_t n = std::min(particles_.size(), pressures_.size());
    std::copy(pressures_.begin() + static_cast<std::ptrdiff_t>(n), pressures_.end(), out + n);
    if (n) copy_field(3, out);
}

// SPHEngine::step (src/sph_engine.cpp:93-144)
void SPHEngine::step(float dt) {
    if (!initialized_ || particles_.size() == 0) return;
    sync_to_device();
    check(sphx_step(gpu_, dt), "sphx_step");
    ++step_count_;
    host_stale_ = true;
}

void SPHEngine::run_steps(size_t num_steps, bool adaptive_timestep) {
    for (size_t i = 0; i < num_steps; ++i) step(adaptive_timestep ? 0.0f : params_.timestep);
}

const ParticleSystem& SPHEngine::get_particles() const {
    sync_to_host();
    return particles_;
}

float SPHEngine::get_current_time() const {
    float t = 0.0f, dt = 0.0f;
    check(sphx_get_time(gpu_, &t, &dt), "sphx_get_time");
    return t;
}

// SPHEngine::set_parameters (cpp:152-156): the search radius becomes 2h
void SPHEngine::set_parameters(const SPHParameters& params) {
    params_ = params;
    set_smoothing_length(params.smoothing_length);
}

void SPHEngine::set_gravity(float gravity) {
    params_.gravity = gravity;
    push_params();
}

void SPHEngine::set_viscosity(float viscosity) {
    params_.viscosity = viscosity;
    push_params();
}

// SPHEngine::set_smoothing_length (cpp:158-163)
void SPHEngine::set_smoothing_length(float h) {
    params_.smoothing_length = h;
    params_.neighbor_search_radius = 2.0f * h;
    push_params();
}

void SPHEngine::set_kernel_type(KernelType type) {
    const int k = static_cast<int>(type);
    if (k < SPHX_KERNEL_CUBIC_SPLINE || k > SPHX_KERNEL_GAUSSIAN)
        throw std::invalid_argument("Unknown kernel type");
    check(sphx_set_kernel(gpu_, k), "sphx_set_kernel");
    kernel_type_ = type;
}

void SPHEngine::set_boundaries(float xmin, float xmax, float ymin, float ymax, float zmin,
                               float zmax) {
    params_.bounds.xmin = xmin;
    params_.bounds.xmax = xmax;
    params_.bounds.ymin = ymin;
    params_.bounds.ymax = ymax;
    params_.bounds.zmin = zmin;
    params_.bounds.zmax = zmax;
    push_params();
}

const SPHEngine::PerformanceStats& SPHEngine::get_performance_stats() const {
    sphx_stats s;
    const int rc = sphx_get_stats(gpu_, &s);
    if (rc != SPHX_OK && rc != SPHX_ERR_DOMAIN) check(rc, "sphx_get_stats");
    perf_stats_.total_time = s.total_time;
    perf_stats_.neighbor_search_time = s.neighbor_search_time;
    perf_stats_.density_computation_time = s.density_computation_time;
    perf_stats_.force_computation_time = s.force_computation_time;
    perf_stats_.integration_time = s.integration_time;
    perf_stats_.max_neighbors = static_cast<size_t>(s.max_neighbors);
    perf_stats_.total_neighbor_queries = static_cast<size_t>(s.total_neighbor_queries);
    return perf_stats_;
}

void SPHEngine::reset_performance_stats() {
    perf_stats_ = PerformanceStats{};
    check(sphx_reset_stats(gpu_), "sphx_reset_stats");
}

// compute_conservation_errors (cpp:178-185)
void SPHEngine::compute_conservation_errors(float& mass_error, float& energy_error) const {
    const float total_mass = get_total_mass();
    const float initial_mass = static_cast<float>(particles_.size()) * params_.particle_mass;
    mass_error = std::abs(total_mass - initial_mass) / initial_mass;
    energy_error = 0.0f;
}

// get_total_mass (cpp:187-190): sum of the densities in float, times h^3
float SPHEngine::get_total_mass() const {
    sync_to_host();
    float s = 0.0f;
    const size_t n = std::min(particles_.size(), densities_.size());
    for (size_t i = 0; i < n; ++i) s = s + densities_[i];
    const float h = params_.smoothing_length;
    return s * (h * h * h);
}

// get_total_energy (cpp:192-200): kinetic energy in float
float SPHEngine::get_total_energy() const {
    sync_to_host();
    float ke = 0.0f;
    for (size_t i = 0; i < particles_.size(); ++i) {
        const Particle& p = particles_[i];
        const float speed_sq = glm::dot(p.velocity, p.velocity);
        ke += 0.5f * p.mass * speed_sq;
    }
    return ke;
}

std::vector<glm::vec3> SPHEngine::get_positions() const {
    std::vector<glm::vec3> out(particles_.size());
    if (!out.empty()) copy_positions(&out[0].x);
    return out;
}

std::vector<glm::vec3> SPHEngine::get_velocities() const {
    std::vector<glm::vec3> out(particles_.size());
    if (!out.empty()) copy_velocities(&out[0].x);
    return out;
}

std::vector<float> SPHEngine::get_densities() const {
    std::vector<float> out(densities_.size());
    if (!out.empty()) copy_densities(out.data());
    return out;
}

std::vector<float> SPHEngine::get_pressures() const {
    std::vector<float> out(pressures_.size());
    if (!out.empty()) copy_pressures(out.data());
    return out;
}

std::vector<double> SPHEngine::get_conservation_sums() const {
    sphx_stats s;
    check(sphx_get_stats(gpu_, &s), "sphx_get_stats");
    return {s.sum_mass, s.momentum[0], s.momentum[1], s.momentum[2], s.kinetic_energy,
            s.potential_energy, s.sum_density};
}

// validate_simulation (cpp:355-365)
void SPHEngine::validate_simulation() const {
    sync_to_host();
    if (!utils::validate_particle_setup(std::vector<Particle>(particles_.begin(), particles_.end())))
        std::cerr << "Warning: Particle setup validation failed\n";
    const float avg = utils::compute_average_neighbors(*this);
    if (avg < 20.0f || avg > 80.0f)
        std::cerr << "Warning: Average neighbor count (" << avg
                  << ") may affect simulation stability\n";
}

namespace equations {

float compute_density(size_t i, const std::vector<size_t>& neighbors,
                      const ParticleSystem& particles, const Kernel& kernel) {
    const Particle& self = particles[i];
    float rho = self.mass * kernel.W(glm::vec3(0.0f));
    for (const size_t j : neighbors) {
        if (j == i) continue;
        const Particle& other = particles[j];
        rho += other.mass * kernel.W(self.position - other.position);
    }
    return rho;
}

float compute_pressure(float density, float rest_density, float gas_constant) {
    return gas_constant * (density - rest_density);
}

glm::vec3 compute_pressure_force(size_t i, const std::vector<size_t>& neighbors,
                                 const ParticleSystem& particles, const Kernel& kernel,
                                 const std::vector<float>& pressures,
                                 const std::vector<float>& densities) {
    const Particle& self = particles[i];
    glm::vec3 f(0.0f);
    for (const size_t j : neighbors) {
        if (j == i) continue;
        const Particle& other = particles[j];
        const glm::vec3 r = self.position - other.position;
        if (glm::length(r) < 1e-6f) continue;  // coincident pair: no direction
        const float shared = (pressures[i] + pressures[j]) / (2.0f * densities[j]);
        f -= other.mass * shared * kernel.gradW(r);
    }
    return f;
}

glm::vec3 compute_viscosity_force(size_t i, const std::vector<size_t>& neighbors,
                                  const ParticleSystem& particles, const Kernel& kernel,
                                  float viscosity, const std::vector<float>& densities) {
    const Particle& self = particles[i];
    glm::vec3 f(0.0f);
    for (const size_t j : neighbors) {
        if (j == i) continue;
        const Particle& other = particles[j];
        const glm::vec3 r = self.position - other.position;
        const glm::vec3 dv = other.velocity - self.velocity;
        const float lap = kernel.laplacianW(r);
        f += (other.mass / densities[j]) * viscosity * dv * lap;
    }
    return f;
}

glm::vec3 compute_external_forces(float gravity) { return glm::vec3(0.0f, gravity, 0.0f); }

glm::vec3 compute_acceleration(const glm::vec3& pressure_force,
                               const glm::vec3& viscosity_force,
                               const glm::vec3& external_force, float particle_mass) {
    return (pressure_force + viscosity_force + external_force * particle_mass) / particle_mass;
}

}  // namespace equations

namespace utils {

// create_dam_break_setup (cpp:450-487): a boundary box shell, then a fluid block
std::vector<Particle> create_dam_break_setup(const glm::vec3& dam_size,
                                             const glm::vec3& fluid_size, float spacing,
                                             const SPHParameters& params) {
    std::vector<Particle> out =
        create_boundary_box(glm::vec3(0.0f, dam_size.y / 2.0f, 0.0f), dam_size, spacing,
                            params.particle_mass);
    for (Particle& p : out) {
        p.type = ParticleType::BOUNDARY;
        p.velocity = glm::vec3(0.0f);
        p.color = glm::vec3(0.5f, 0.5f, 0.5f);
    }
    std::vector<Particle> fluid = create_fluid_block(
        glm::vec3(-dam_size.x / 2.0f + fluid_size.x / 2.0f, fluid_size.y / 2.0f, 0.0f),
        fluid_size, spacing, params.particle_mass);
    for (Particle& p : fluid) {
        p.type = ParticleType::FLUID;
        p.color = glm::vec3(0.0f, 0.5f, 1.0f);
    }
    out.insert(out.end(), fluid.begin(), fluid.end());
    return out;
}

// create_fluid_drop_setup (cpp:489-514): lattice points inside a sphere
std::vector<Particle> create_fluid_drop_setup(const glm::vec3& center, float radius,
                                              float spacing, const SPHParameters& params) {
    std::vector<Particle> out;
    const int per_dim = static_cast<int>(2.0f * radius / spacing);
    const glm::vec3 start = center - glm::vec3(radius);
    for (int i = 0; i < per_dim; ++i)
        for (int j = 0; j < per_dim; ++j)
            for (int k = 0; k < per_dim; ++k) {
                const glm::vec3 pos =
                    start + glm::vec3(static_cast<float>(i) * spacing,
                                      static_cast<float>(j) * spacing,
                                      static_cast<float>(k) * spacing);
                const glm::vec3 d = pos - center;
                if (glm::dot(d, d) <= radius * radius) {
                    Particle p(pos, params.particle_mass, ParticleType::FLUID);
                    p.color = glm::vec3(0.0f, 0.7f, 1.0f);
                    out.push_back(p);
                }
            }
    return out;
}

// create_granular_flow_setup (cpp:516-552): a box shell, then a pile of SOLID particles
std::vector<Particle> create_granular_flow_setup(const glm::vec3& pile_size,
                                                 const glm::vec3& domain_size, float spacing,
                                                 const SPHParameters& params) {
    std::vector<Particle> out =
        create_boundary_box(glm::vec3(0.0f, domain_size.y / 2.0f, 0.0f), domain_size,
                            spacing, params.particle_mass);
    for (Particle& p : out) {
        p.type = ParticleType::BOUNDARY;
        p.color = glm::vec3(0.4f, 0.4f, 0.4f);
    }
    std::vector<Particle> pile =
        create_fluid_block(glm::vec3(0.0f, pile_size.y / 2.0f + spacing, 0.0f), pile_size,
                           spacing, params.particle_mass);
    for (Particle& p : pile) {
        p.type = ParticleType::SOLID;
        p.color = glm::vec3(0.8f, 0.6f, 0.2f);
    }
    out.insert(out.end(), pile.begin(), pile.end());
    return out;
}

// validate_particle_setup (cpp:554-569): O(N^2) overlap check
bool validate_particle_setup(const std::vector<Particle>& particles) {
    if (particles.empty()) return false;
    for (size_t i = 0; i < particles.size(); ++i)
        for (size_t j = i + 1; j < particles.size(); ++j) {
            const glm::vec3 d = particles[i].position - particles[j].position;
            if (glm::dot(d, d) < 1e-8f) {
                std::cerr << "Warning: Overlapping particles detected\n";
                return false;
            }
        }
    return true;
}

// compute_average_neighbors (cpp:571-578): the reference returns a fixed estimate
float compute_average_neighbors(const SPHEngine& engine) {
    if (engine.get_particles().size() == 0) return 0.0f;
    return 50.0f;
}

}  // namespace utils

}  // namespace sph
