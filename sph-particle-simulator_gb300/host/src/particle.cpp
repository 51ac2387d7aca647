// Host particle container and initial-condition generators of the drop-in engine
// (reference semantics: src/particle.cpp:14-229).  Built with -ffp-contract=off so that
// generated positions round exactly like the reference's.
#include "particle.h"

#include <algorithm>
#include <iostream>
#include <random>

namespace sph {

ParticleSystem::ParticleSystem(size_t capacity) : capacity_(capacity) {
    particles_.reserve(capacity_);
}

void ParticleSystem::reserve(size_t capacity) {
    capacity_ = capacity;
    particles_.reserve(capacity_);
}

void ParticleSystem::resize(size_t size) { particles_.resize(size); }

void ParticleSystem::clear() { particles_.clear(); }

void ParticleSystem::add_particle(const Particle& particle) {
    if (particles_.size() >= capacity_) {
        std::cerr << "Warning: Particle capacity exceeded\n";
        return;
    }
    particles_.push_back(particle);
    particles_.back().id = static_cast<int>(particles_.size() - 1);
}

void ParticleSystem::add_particles(const std::vector<Particle>& new_particles) {
    for (const Particle& p : new_particles) add_particle(p);
}

void ParticleSystem::remove_particle(size_t index) {
    if (index >= particles_.size()) return;
    particles_.erase(particles_.begin() + static_cast<std::ptrdiff_t>(index));
    for (size_t i = index; i < particles_.size(); ++i) particles_[i].id = static_cast<int>(i);
}

void ParticleSystem::remove_particles(const std::vector<size_t>& indices) {
    std::vector<size_t> order(indices);
    std::sort(order.begin(), order.end(), [](size_t a, size_t b) { return a > b; });
    for (size_t index : order)
        if (index < particles_.size())
            particles_.erase(particles_.begin() + static_cast<std::ptrdiff_t>(index));
    for (size_t i = 0; i < particles_.size(); ++i) particles_[i].id = static_cast<int>(i);
}

// The getters copy one field of every particle out of the AoS store (in parallel for
// large sets: they run after every step of a host-side loop).
template <class T, class F>
static std::vector<T> gather(const std::vector<Particle>& ps, F field) {
    std::vector<T> out(ps.size());
    const long long n = static_cast<long long>(ps.size());
#pragma omp parallel for schedule(static) if (n > 65536)
    for (long long i = 0; i < n; ++i) out[i] = field(ps[static_cast<size_t>(i)]);
    return out;
}

std::vector<glm::vec3> ParticleSystem::get_positions() const {
    return gather<glm::vec3>(particles_, [](const Particle& p) { return p.position; });
}

std::vector<glm::vec3> ParticleSystem::get_velocities() const {
    return gather<glm::vec3>(particles_, [](const Particle& p) { return p.velocity; });
}

std::vector<float> ParticleSystem::get_densities() const {
    return gather<float>(particles_, [](const Particle& p) { return p.density; });
}

std::vector<float> ParticleSystem::get_pressures() const {
    return gather<float>(particles_, [](const Particle& p) { return p.pressure; });
}

void ParticleSystem::set_mass(float mass) {
    for (Particle& p : particles_) p.mass = mass;
}

void ParticleSystem::set_viscosity(float viscosity) {
    for (Particle& p : particles_) p.viscosity = viscosity;
}

void ParticleSystem::set_temperature(float temperature) {
    for (Particle& p : particles_) p.temperature = temperature;
}

void ParticleSystem::apply_boundary_conditions(float xmin, float xmax, float ymin, float ymax,
                                               float zmin, float zmax) {
    const float lo[3] = {xmin, ymin, zmin}, hi[3] = {xmax, ymax, zmax};
    for (Particle& p : particles_) {
        for (int a = 0; a < 3; ++a) {
            if (p.position[a] < lo[a]) {
                p.position[a] = lo[a];
                p.velocity[a] *= -0.8f;
            } else if (p.position[a] > hi[a]) {
                p.position[a] = hi[a];
                p.velocity[a] *= -0.8f;
            }
        }
    }
}

glm::vec3 generate_random_position(float xmin, float xmax, float ymin, float ymax, float zmin,
                                   float zmax) {
    static std::mt19937 gen{std::random_device{}()};
    std::uniform_real_distribution<float> dx(xmin, xmax), dy(ymin, ymax), dz(zmin, zmax);
    const float x = dx(gen);
    const float y = dy(gen);
    const float z = dz(gen);
    return glm::vec3(x, y, z);
}

std::vector<Particle> create_fluid_block(const glm::vec3& center, const glm::vec3& size,
                                         float spacing, float mass) {
    const int nx = static_cast<int>(size.x / spacing);
    const int ny = static_cast<int>(size.y / spacing);
    const int nz = static_cast<int>(size.z / spacing);
    const glm::vec3 start = center - size * 0.5f;
    std::vector<Particle> out;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const glm::vec3 offset(static_cast<float>(i) * spacing,
                                       static_cast<float>(j) * spacing,
                                       static_cast<float>(k) * spacing);
                Particle p(start + offset, mass, ParticleType::FLUID);
                p.color = glm::vec3(0.0f, 0.5f + 0.5f * (p.position.y - start.y) / size.y, 1.0f);
                out.push_back(p);
            }
    return out;
}

std::vector<Particle> create_boundary_box(const glm::vec3& center, const glm::vec3& size,
                                          float spacing, float mass) {
    const glm::vec3 start = center - size * 0.5f;
    std::vector<Particle> out;
    // one face: a lattice over axes (u, v) at coordinate `value` on axis w
    auto face = [&](int u, int v, int w, float value) {
        const int nu = static_cast<int>(size[u] / spacing);
        const int nv = static_cast<int>(size[v] / spacing);
        for (int i = 0; i < nu; ++i)
            for (int j = 0; j < nv; ++j) {
                glm::vec3 pos = start;
                pos[u] = start[u] + static_cast<float>(i) * spacing;
                pos[v] = start[v] + static_cast<float>(j) * spacing;
                pos[w] = value;
                Particle p(pos, mass, ParticleType::BOUNDARY);
                p.color = glm::vec3(0.5f, 0.5f, 0.5f);
                out.push_back(p);
            }
    };
    face(0, 1, 2, start.z);           // z = min
    face(0, 1, 2, start.z + size.z);  // z = max
    face(1, 2, 0, start.x);           // x = min
    face(1, 2, 0, start.x + size.x);  // x = max
    face(0, 2, 1, start.y);           // y = min
    face(0, 2, 1, start.y + size.y);  // y = max
    return out;
}

}  // namespace sph
