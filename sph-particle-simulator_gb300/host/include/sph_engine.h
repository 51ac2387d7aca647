// GB300 drop-in for the reference's SPH engine (src/sph_engine.h).
//
// Same namespace, class names, members functions and semantics as the reference's
// SPHParameters / SPHEngine / utils:: (src/sph_engine.h:14-204); SPHEngine::step runs on
// the GPU through the sphx C ABI (include/sphx.h).  The particle set lives on the device;
// the host ParticleSystem is a mirror kept in insertion order and synchronised lazily:
// uploaded before a step when the host side changed (add_particles, clear_particles,
// initialize_*), downloaded when read (get_particles, get_positions, ...).
//
// Differences from the reference, all deliberate:
//  * PerformanceStats is public (the reference declares it private, which makes its own
//    pybind11 module fail to compile, python/bindings.cpp:73).
//  * Its timing fields are device times of the step's phases (CUDA events); the
//    integration phase is fused into the force pass, so integration_time stays 0.
//    max_neighbors / total_neighbor_queries are exact (the reference's are updated
//    without synchronisation inside an OpenMP loop, sph_engine.cpp:350-351).
//  * The kernel classes, create_kernel (kernels.h) and the equations:: free functions are
//    provided for user code as host evaluations with the reference's float operations;
//    step() itself does not call them: its per-pair equations run on the GPU, in the
//    same order.
//  * set_kernel_type / get_kernel_type (new) select the smoothing kernel of the step among
//    the three create_kernel offers.  The reference engine always uses the cubic spline
//    (sph_engine.cpp:17, 23, 162), which stays the default; the choice survives
//    set_smoothing_length and initialize.
//  * Device failures surface as std::runtime_error (the reference has none to report).
#pragma once

#include <cstddef>
#include <memory>
#include <vector>

#include "kernels.h"
#include "particle.h"
#include "spatial_hash.h"

struct sphx_ctx;

namespace sph {

// Simulation parameters (src/sph_engine.h:14-34), same fields, defaults and order.
struct SPHParameters {
    float rest_density = 1000.0f;
    float gas_constant = 2000.0f;
    float viscosity = 0.001f;
    float smoothing_length = 0.02f;
    float particle_mass = 0.001f;
    float timestep = 0.001f;
    float gravity = -9.81f;
    float damping = 0.99f;
    float CFL_factor = 0.4f;

    struct Boundaries {
        float xmin = -1.0f, xmax = 1.0f;
        float ymin = -1.0f, ymax = 1.0f;
        float zmin = -1.0f, zmax = 1.0f;
    } bounds;

    float neighbor_search_radius = 0.04f;
};

class SPHEngine {
   public:
    // Per-phase timers and neighbour statistics (src/sph_engine.h:51-59), public here.
    struct PerformanceStats {
        double total_time = 0.0;
        double neighbor_search_time = 0.0;
        double density_computation_time = 0.0;
        double force_computation_time = 0.0;
        double integration_time = 0.0;
        size_t max_neighbors = 0;
        size_t total_neighbor_queries = 0;
    };

    explicit SPHEngine(size_t max_particles = 1000000);
    ~SPHEngine();
    SPHEngine(const SPHEngine&) = delete;
    SPHEngine& operator=(const SPHEngine&) = delete;

    void initialize(const SPHParameters& params);
    void initialize_dam_break();
    void initialize_fluid_drop();
    void initialize_granular_flow();

    void add_particles(const std::vector<Particle>& particles);
    void clear_particles();

    void step(float dt = 0.0f);  // dt <= 0: adaptive (CFL) timestep
    void run_steps(size_t num_steps, bool adaptive_timestep = true);

    const ParticleSystem& get_particles() const;
    const SPHParameters& get_parameters() const { return params_; }
    float get_current_time() const;
    size_t get_step_count() const { return step_count_; }

    void set_parameters(const SPHParameters& params);
    void set_gravity(float gravity);
    void set_viscosity(float viscosity);
    void set_smoothing_length(float h);
    void set_boundaries(float xmin, float xmax, float ymin, float ymax, float zmin, float zmax);

    // Smoothing kernel of step() (an addition to the reference's API, see above).
    void set_kernel_type(KernelType type);
    KernelType get_kernel_type() const { return kernel_type_; }

    const PerformanceStats& get_performance_stats() const;
    void reset_performance_stats();

    void compute_conservation_errors(float& mass_error, float& energy_error) const;
    float get_total_mass() const;
    float get_total_energy() const;

    std::vector<glm::vec3> get_positions() const;
    std::vector<glm::vec3> get_velocities() const;
    std::vector<float> get_densities() const;   // capacity-length, like the reference
    std::vector<float> get_pressures() const;   // capacity-length, like the reference

    void validate_simulation() const;
    bool is_initialized() const { return initialized_; }

    // GPU-side FP64 conservation sums of the state after the last step: mass, momentum
    // (3), kinetic energy, potential energy (-m g y), sum of densities.
    std::vector<double> get_conservation_sums() const;

    // Copies of the current state into caller arrays, read from the device without
    // refreshing the whole host mirror (what get_positions & co. return, without the
    // intermediate vector): positions / velocities 3 floats per particle (particle_count()
    // particles), densities / pressures the capacity-length arrays of get_densities /
    // get_pressures.  Not in the reference's API; the Python module's getters use them.
    size_t particle_count() const { return particles_.size(); }
    size_t density_count() const { return densities_.size(); }
    void copy_positions(float* out) const;
    void copy_velocities(float* out) const;
    void copy_densities(float* out) const;
    void copy_pressures(float* out) const;

   private:
    void push_params();
    void sync_to_host() const;   // device -> host mirror, when the device is newer
    void sync_to_device();       // host mirror -> device, when the host changed
    void host_will_change();     // call before mutating the host mirror
    void replace_particles(const std::vector<Particle>& ps);
    void stage_append(size_t from);  // mirror particles [from, size) -> upload region
    void copy_field(int field, float* out) const;

    float* stage() const;        // pinned transfer buffers (15 floats per particle)

    mutable ParticleSystem particles_;
    mutable float* stage_ = nullptr;   // x, v, m (upload) | rho, P, x, v (download)
    size_t staged_ = 0;                // particles the upload region holds
    bool stage_current_ = false;       // the upload region equals the mirror's first staged_
    SPHParameters params_;
    KernelType kernel_type_ = KernelType::CUBIC_SPLINE;
    sphx_ctx* gpu_ = nullptr;
    size_t step_count_ = 0;
    bool initialized_ = false;
    mutable bool host_stale_ = false;  // the device holds a newer state than the mirror
    bool device_dirty_ = true;         // the mirror changed since the last upload
    mutable std::vector<float> densities_;
    mutable std::vector<float> pressures_;
    mutable PerformanceStats perf_stats_;
};

// Integration methods (src/sph_engine.h:144-148); the step always uses leapfrog.
enum class IntegrationMethod { EULER, VERLET, LEAPFROG };

// The SPH equations of one particle (src/sph_engine.h:150-179), evaluated on the host with
// the reference's float operations in its order, so that user code calling them gets the
// reference's numbers.  `neighbors` lists indices into `particles` (self included or not:
// i itself is skipped).
namespace equations {

// rho_i = m_i W(0) + sum_{j != i} m_j W(r_ij)
float compute_density(size_t i, const std::vector<size_t>& neighbors,
                      const ParticleSystem& particles, const Kernel& kernel);
// P = k (rho - rho0)
float compute_pressure(float density, float rest_density, float gas_constant);
// -sum_{j != i, |r_ij| >= 1e-6} m_j (P_i + P_j) / (2 rho_j) grad W(r_ij)
glm::vec3 compute_pressure_force(size_t i, const std::vector<size_t>& neighbors,
                                 const ParticleSystem& particles, const Kernel& kernel,
                                 const std::vector<float>& pressures,
                                 const std::vector<float>& densities);
// sum_{j != i} (m_j / rho_j) mu (v_j - v_i) laplacian W(r_ij)
glm::vec3 compute_viscosity_force(size_t i, const std::vector<size_t>& neighbors,
                                  const ParticleSystem& particles, const Kernel& kernel,
                                  float viscosity, const std::vector<float>& densities);
// (0, g, 0)
glm::vec3 compute_external_forces(float gravity);
// (F_p + F_v + F_ext m) / m
glm::vec3 compute_acceleration(const glm::vec3& pressure_force,
                               const glm::vec3& viscosity_force,
                               const glm::vec3& external_force, float particle_mass);

}  // namespace equations

namespace utils {

// Scene generators (src/sph_engine.cpp:450-552).
std::vector<Particle> create_dam_break_setup(const glm::vec3& dam_size,
                                             const glm::vec3& fluid_size, float spacing,
                                             const SPHParameters& params);
std::vector<Particle> create_fluid_drop_setup(const glm::vec3& center, float radius,
                                              float spacing, const SPHParameters& params);
std::vector<Particle> create_granular_flow_setup(const glm::vec3& pile_size,
                                                 const glm::vec3& domain_size, float spacing,
                                                 const SPHParameters& params);

bool validate_particle_setup(const std::vector<Particle>& particles);
float compute_average_neighbors(const SPHEngine& engine);

}  // namespace utils

}  // namespace sph
