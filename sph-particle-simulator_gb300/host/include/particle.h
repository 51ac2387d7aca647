// Particle record and host-side particle container of the GB300 drop-in engine.
//
// Same types, fields, constructors and member functions as the reference's particle.h
// (src/particle.h:9-105), so code written against the reference compiles unchanged.  In
// the drop-in, ParticleSystem is the host mirror of the particle set: SPHEngine keeps it
// in insertion order and synchronises it with the device state when it is read.
#pragma once

#include <glm/glm.hpp>
#include <memory>
#include <vector>

namespace sph {

// Particle types (src/particle.h:10-14).  The step treats all types alike, as the
// reference does.
enum class ParticleType { FLUID, BOUNDARY, SOLID };

// Particle record (src/particle.h:17-49).
struct Particle {
    glm::vec3 position;
    glm::vec3 velocity;
    glm::vec3 acceleration;  // never written by the step (the reference keeps its
                             // accelerations in a separate engine buffer)
    float density;
    float pressure;
    float mass;
    ParticleType type;
    float temperature;
    float viscosity;
    glm::vec3 color;
    int id;

    Particle()
        : position(0.0f), velocity(0.0f), acceleration(0.0f), density(0.0f), pressure(0.0f),
          mass(1.0f), type(ParticleType::FLUID), temperature(293.15f), viscosity(0.001f),
          color(0.0f, 0.5f, 1.0f), id(-1) {}

    Particle(const glm::vec3& pos, float m = 1.0f, ParticleType t = ParticleType::FLUID)
        : position(pos), velocity(0.0f), acceleration(0.0f), density(0.0f), pressure(0.0f),
          mass(m), type(t), temperature(293.15f), viscosity(0.001f), color(0.0f, 0.5f, 1.0f),
          id(-1) {}
};

// Container with a capacity cap (src/particle.h:52-100): particles beyond the capacity
// are dropped with a warning on stderr; id = insertion index.
class ParticleSystem {
   private:
    std::vector<Particle> particles_;
    size_t capacity_;

   public:
    explicit ParticleSystem(size_t capacity = 1000000);
    ~ParticleSystem() = default;

    void reserve(size_t capacity);
    void resize(size_t size);
    void clear();

    Particle& operator[](size_t index) { return particles_[index]; }
    const Particle& operator[](size_t index) const { return particles_[index]; }
    size_t size() const { return particles_.size(); }
    size_t capacity() const { return capacity_; }
    bool empty() const { return particles_.empty(); }

    auto begin() { return particles_.begin(); }
    auto end() { return particles_.end(); }
    auto begin() const { return particles_.cbegin(); }
    auto end() const { return particles_.cend(); }

    void add_particle(const Particle& particle);
    void add_particles(const std::vector<Particle>& new_particles);

    void remove_particle(size_t index);
    void remove_particles(const std::vector<size_t>& indices);

    std::vector<glm::vec3> get_positions() const;
    std::vector<glm::vec3> get_velocities() const;
    std::vector<float> get_densities() const;
    std::vector<float> get_pressures() const;

    void set_mass(float mass);
    void set_viscosity(float viscosity);
    void set_temperature(float temperature);

    // Wall clamp with restitution -0.8 on the host copy (src/particle.cpp:122-153).  The
    // engine's step applies the same rule on the GPU.
    void apply_boundary_conditions(float xmin, float xmax, float ymin, float ymax, float zmin,
                                   float zmax);
};

glm::vec3 generate_random_position(float xmin, float xmax, float ymin, float ymax, float zmin,
                                   float zmax);
// Lattice block and six-face box shell generators (src/particle.cpp:156-229).
std::vector<Particle> create_fluid_block(const glm::vec3& center, const glm::vec3& size,
                                         float spacing, float mass = 1.0f);
std::vector<Particle> create_boundary_box(const glm::vec3& center, const glm::vec3& size,
                                          float spacing, float mass = 1.0f);

}  // namespace sph
