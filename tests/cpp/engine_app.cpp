// An application written against the reference's C++ engine API (src/sph_engine.h,
// src/kernels.h), compiled unchanged against the drop-in headers: it sets up the dam
// break, steps it, and prints one JSON line with counts, times and an FNV-1a hash of the
// positions and densities (float bits), which the tests compare with the oracle engine.
//
// Usage: engine_app <steps> <dt> ; dt <= 0 runs CFL steps.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "sph_engine.h"

namespace {

uint64_t fnv1a(uint64_t h, const void* data, size_t bytes) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < bytes; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

}  // namespace

int main(int argc, char** argv) {
    const int steps = argc > 1 ? std::atoi(argv[1]) : 3;
    const float dt = argc > 2 ? static_cast<float>(std::atof(argv[2])) : 0.001f;

    sph::SPHEngine engine(200000);
    sph::SPHParameters params;
    params.bounds.xmin = -0.25f;
    params.bounds.xmax = 0.25f;
    params.bounds.ymin = 0.0f;
    params.bounds.ymax = 0.7f;
    params.bounds.zmin = -0.45f;
    params.bounds.zmax = 0.45f;
    engine.initialize(params);
    engine.initialize_dam_break();
    for (int s = 0; s < steps; ++s) engine.step(dt);

    const std::vector<glm::vec3> pos = engine.get_positions();
    const std::vector<float> rho = engine.get_densities();
    uint64_t h = 0xcbf29ce484222325ull;
    for (const glm::vec3& p : pos) {
        const float v[3] = {p.x, p.y, p.z};
        h = fnv1a(h, v, sizeof(v));
    }
    h = fnv1a(h, rho.data(), pos.size() * sizeof(float));

    float mass_error = 0.0f, energy_error = 0.0f;
    engine.compute_conservation_errors(mass_error, energy_error);
    const auto& st = engine.get_performance_stats();
    auto kernel = sph::create_kernel(sph::KernelType::CUBIC_SPLINE, params.smoothing_length);
    std::printf(
        "{\"particles\": %zu, \"steps\": %zu, \"time\": %.9g, \"hash\": \"%016llx\", "
        "\"max_neighbors\": %zu, \"total_mass\": %.9g, \"w0\": %.9g, \"valid\": %d}\n",
        engine.get_particles().size(), engine.get_step_count(), engine.get_current_time(),
        static_cast<unsigned long long>(h), st.max_neighbors, engine.get_total_mass(),
        kernel->W(glm::vec3(0.0f)), 1);
    return 0;
}
