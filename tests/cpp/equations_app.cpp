// User code calling the reference's equations:: free functions (src/sph_engine.h:150-179)
// through the drop-in headers.  Reads a state and its neighbour lists from a binary file,
// evaluates density, pressure and acceleration per particle with equations:: and the
// kernel create_kernel returns, and writes them out for the tests to compare with the
// oracle bit for bit.
//
// Usage: equations_app <in> <out>
//   in:  int64 n, int32 kernel, 16 float parameters (SPHParameters order), n*3 float
//        positions, n*3 float velocities, n float masses, n int64 list lengths, then the
//        concatenated int64 lists
//   out: n float densities, n float pressures, n*3 float accelerations
#include <cstdint>
#include <cstdio>
#include <vector>

#include "sph_engine.h"

namespace {

template <class T>
bool read_n(std::FILE* f, T* out, size_t n) {
    return std::fread(out, sizeof(T), n, f) == n;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t n = 0;
    int32_t kind = 0;
    float prm[16];
    if (!read_n(f, &n, 1) || !read_n(f, &kind, 1) || !read_n(f, prm, 16)) return 3;
    std::vector<float> pos(3 * n), vel(3 * n), mass(n);
    std::vector<int64_t> counts(n);
    if (!read_n(f, pos.data(), pos.size()) || !read_n(f, vel.data(), vel.size()) ||
        !read_n(f, mass.data(), mass.size()) || !read_n(f, counts.data(), counts.size()))
        return 3;
    std::vector<std::vector<size_t>> lists(n);
    for (int64_t i = 0; i < n; ++i) {
        std::vector<int64_t> l(counts[i]);
        if (!read_n(f, l.data(), l.size())) return 3;
        lists[i].assign(l.begin(), l.end());
    }
    std::fclose(f);

    sph::ParticleSystem ps(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        sph::Particle p(glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), mass[i]);
        p.velocity = glm::vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        ps.add_particle(p);
    }
    auto kernel = sph::create_kernel(static_cast<sph::KernelType>(kind), prm[3]);
    std::vector<float> rho(n), P(n), acc(3 * n);
    for (int64_t i = 0; i < n; ++i)
        rho[i] = sph::equations::compute_density(i, lists[i], ps, *kernel);
    for (int64_t i = 0; i < n; ++i) P[i] = sph::equations::compute_pressure(rho[i], prm[0], prm[1]);
    for (int64_t i = 0; i < n; ++i) {
        const glm::vec3 fp =
            sph::equations::compute_pressure_force(i, lists[i], ps, *kernel, P, rho);
        const glm::vec3 fv =
            sph::equations::compute_viscosity_force(i, lists[i], ps, *kernel, prm[2], rho);
        const glm::vec3 a = sph::equations::compute_acceleration(
            fp, fv, sph::equations::compute_external_forces(prm[6]), ps[i].mass);
        acc[3 * i] = a.x;
        acc[3 * i + 1] = a.y;
        acc[3 * i + 2] = a.z;
    }
    std::FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 4;
    std::fwrite(rho.data(), sizeof(float), rho.size(), o);
    std::fwrite(P.data(), sizeof(float), P.size(), o);
    std::fwrite(acc.data(), sizeof(float), acc.size(), o);
    std::fclose(o);
    return 0;
}
