// pybind11 module `sph`: the reference's Python API (python/bindings.cpp:8-166) over the
// GB300 drop-in engine, same class, method and argument names.
//
// Differences from the reference's module, all additions or fixes:
//  * it compiles (PerformanceStats is public in the drop-in);
//  * glm::vec3 is registered as sph.vec3 (x, y, z; constructible from three floats or a
//    3-sequence), so Particle.position & co. work from Python -- the reference binds
//    them without a type for glm::vec3;
//  * SPHParameters also exposes CFL_factor, neighbor_search_radius and the six bounds;
//  * Simulator.add_particles_array(pos, vel, mass) takes numpy arrays directly, and
//    Simulator.get_conservation_sums() returns the GPU's FP64 sums;
//  * sph.SpatialHash binds the GPU-backed spatial hash.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstring>
#include <stdexcept>

#include "sph_engine.h"

namespace py = pybind11;

namespace {

py::array_t<float> vec3_array(const std::vector<glm::vec3>& v) {
    static_assert(sizeof(glm::vec3) == 3 * sizeof(float), "glm::vec3 is three packed floats");
    py::array_t<float> out({static_cast<py::ssize_t>(v.size()), static_cast<py::ssize_t>(3)});
    if (!v.empty()) std::memcpy(out.mutable_data(), v.data(), v.size() * sizeof(glm::vec3));
    return out;
}

py::array_t<float> float_array(const std::vector<float>& v) {
    py::array_t<float> out(static_cast<py::ssize_t>(v.size()));
    std::copy(v.begin(), v.end(), out.mutable_data());
    return out;
}

glm::vec3 vec3_from(const py::array_t<float, py::array::c_style | py::array::forcecast>& a,
                    const char* what) {
    if (a.size() != 3) throw std::invalid_argument(std::string(what) + " must be a 3D vector");
    return glm::vec3(a.at(0), a.at(1), a.at(2));
}

}  // namespace

PYBIND11_MODULE(sph, m) {
    m.doc() = "SPH Particle Simulator - Python bindings (GB300 step)";

    py::class_<glm::vec3>(m, "vec3")
        .def(py::init<>())
        .def(py::init<float, float, float>())
        .def(py::init([](const py::sequence& s) {
            if (py::len(s) != 3) throw std::invalid_argument("vec3 needs 3 components");
            return glm::vec3(s[0].cast<float>(), s[1].cast<float>(), s[2].cast<float>());
        }))
        .def_readwrite("x", &glm::vec3::x)
        .def_readwrite("y", &glm::vec3::y)
        .def_readwrite("z", &glm::vec3::z)
        .def("__len__", [](const glm::vec3&) { return 3; })
        .def("__getitem__", [](const glm::vec3& v, int i) {
            if (i < 0 || i > 2) throw py::index_error();
            return v[i];
        })
        .def("__repr__", [](const glm::vec3& v) {
            return "vec3(" + std::to_string(v.x) + ", " + std::to_string(v.y) + ", " +
                   std::to_string(v.z) + ")";
        });
    py::implicitly_convertible<py::sequence, glm::vec3>();

    py::class_<sph::SPHParameters>(m, "SPHParameters")
        .def(py::init<>())
        .def_readwrite("rest_density", &sph::SPHParameters::rest_density)
        .def_readwrite("gas_constant", &sph::SPHParameters::gas_constant)
        .def_readwrite("viscosity", &sph::SPHParameters::viscosity)
        .def_readwrite("smoothing_length", &sph::SPHParameters::smoothing_length)
        .def_readwrite("particle_mass", &sph::SPHParameters::particle_mass)
        .def_readwrite("timestep", &sph::SPHParameters::timestep)
        .def_readwrite("gravity", &sph::SPHParameters::gravity)
        .def_readwrite("damping", &sph::SPHParameters::damping)
        .def_readwrite("CFL_factor", &sph::SPHParameters::CFL_factor)
        .def_readwrite("neighbor_search_radius", &sph::SPHParameters::neighbor_search_radius)
        .def_property(
            "bounds",
            [](const sph::SPHParameters& p) {
                return py::make_tuple(p.bounds.xmin, p.bounds.xmax, p.bounds.ymin, p.bounds.ymax,
                                      p.bounds.zmin, p.bounds.zmax);
            },
            [](sph::SPHParameters& p, const std::vector<float>& b) {
                if (b.size() != 6) throw std::invalid_argument("bounds has 6 values");
                p.bounds.xmin = b[0];
                p.bounds.xmax = b[1];
                p.bounds.ymin = b[2];
                p.bounds.ymax = b[3];
                p.bounds.zmin = b[4];
                p.bounds.zmax = b[5];
            });

    py::enum_<sph::ParticleType>(m, "ParticleType")
        .value("FLUID", sph::ParticleType::FLUID)
        .value("BOUNDARY", sph::ParticleType::BOUNDARY)
        .value("SOLID", sph::ParticleType::SOLID);

    // smoothing kernels (kernels.h; the reference's module does not bind them)
    py::enum_<sph::KernelType>(m, "KernelType")
        .value("CUBIC_SPLINE", sph::KernelType::CUBIC_SPLINE)
        .value("WENDLAND_C2", sph::KernelType::WENDLAND_C2)
        .value("GAUSSIAN", sph::KernelType::GAUSSIAN);

    py::class_<sph::Kernel>(m, "Kernel")
        .def("W", &sph::Kernel::W)
        .def("gradW", &sph::Kernel::gradW)
        .def("laplacianW", &sph::Kernel::laplacianW)
        .def("get_smoothing_length", &sph::Kernel::get_smoothing_length)
        .def("set_smoothing_length", &sph::Kernel::set_smoothing_length)
        .def("get_support_radius", &sph::Kernel::get_support_radius);

    m.def("create_kernel", &sph::create_kernel, py::arg("type"), py::arg("smoothing_length"));

    py::class_<sph::Particle>(m, "Particle")
        .def(py::init<>())
        .def(py::init<const glm::vec3&, float, sph::ParticleType>(), py::arg("position"),
             py::arg("mass") = 1.0f, py::arg("type") = sph::ParticleType::FLUID)
        .def_readwrite("position", &sph::Particle::position)
        .def_readwrite("velocity", &sph::Particle::velocity)
        .def_readwrite("acceleration", &sph::Particle::acceleration)
        .def_readwrite("density", &sph::Particle::density)
        .def_readwrite("pressure", &sph::Particle::pressure)
        .def_readwrite("mass", &sph::Particle::mass)
        .def_readwrite("type", &sph::Particle::type)
        .def_readwrite("temperature", &sph::Particle::temperature)
        .def_readwrite("viscosity", &sph::Particle::viscosity)
        .def_readwrite("color", &sph::Particle::color)
        .def_readonly("id", &sph::Particle::id);

    py::class_<sph::ParticleSystem>(m, "ParticleSystem")
        .def("size", &sph::ParticleSystem::size)
        .def("capacity", &sph::ParticleSystem::capacity)
        .def("empty", &sph::ParticleSystem::empty)
        .def("__len__", &sph::ParticleSystem::size)
        .def("__getitem__",
             [](const sph::ParticleSystem& ps, size_t i) {
                 if (i >= ps.size()) throw py::index_error();
                 return ps[i];
             })
        .def("get_positions", [](const sph::ParticleSystem& ps) { return vec3_array(ps.get_positions()); })
        .def("get_velocities", [](const sph::ParticleSystem& ps) { return vec3_array(ps.get_velocities()); })
        .def("get_densities", [](const sph::ParticleSystem& ps) { return float_array(ps.get_densities()); })
        .def("get_pressures", [](const sph::ParticleSystem& ps) { return float_array(ps.get_pressures()); });

    using PS = sph::SPHEngine::PerformanceStats;
    py::class_<PS>(m, "PerformanceStats")
        .def_readonly("total_time", &PS::total_time)
        .def_readonly("neighbor_search_time", &PS::neighbor_search_time)
        .def_readonly("density_computation_time", &PS::density_computation_time)
        .def_readonly("force_computation_time", &PS::force_computation_time)
        .def_readonly("integration_time", &PS::integration_time)
        .def_readonly("max_neighbors", &PS::max_neighbors)
        .def_readonly("total_neighbor_queries", &PS::total_neighbor_queries);

    py::class_<sph::SPHEngine>(m, "Simulator")
        .def(py::init<size_t>(), py::arg("max_particles") = 1000000)
        .def("initialize", &sph::SPHEngine::initialize, py::arg("params"))
        .def("initialize_dam_break", &sph::SPHEngine::initialize_dam_break)
        .def("initialize_fluid_drop", &sph::SPHEngine::initialize_fluid_drop)
        .def("initialize_granular_flow", &sph::SPHEngine::initialize_granular_flow)
        .def("add_particles", &sph::SPHEngine::add_particles)
        .def("add_particles_array",
             [](sph::SPHEngine& e, py::array_t<float, py::array::c_style | py::array::forcecast> pos,
                py::object vel, py::array_t<float, py::array::c_style | py::array::forcecast> mass) {
                 if (pos.ndim() != 2 || pos.shape(1) != 3) throw std::invalid_argument("pos is (n, 3)");
                 const size_t n = static_cast<size_t>(pos.shape(0));
                 if (static_cast<size_t>(mass.size()) != n) throw std::invalid_argument("mass is (n,)");
                 py::array_t<float, py::array::c_style | py::array::forcecast> v;
                 if (!vel.is_none()) {
                     v = vel.cast<py::array_t<float, py::array::c_style | py::array::forcecast>>();
                     if (static_cast<size_t>(v.size()) != 3 * n) throw std::invalid_argument("vel is (n, 3)");
                 }
                 std::vector<sph::Particle> ps(n);
                 const float* p = pos.data();
                 const float* mm = mass.data();
                 for (size_t i = 0; i < n; ++i) {
                     ps[i] = sph::Particle(glm::vec3(p[3 * i], p[3 * i + 1], p[3 * i + 2]), mm[i]);
                     if (!vel.is_none())
                         ps[i].velocity = glm::vec3(v.data()[3 * i], v.data()[3 * i + 1], v.data()[3 * i + 2]);
                 }
                 e.add_particles(ps);
             },
             py::arg("pos"), py::arg("vel") = py::none(), py::arg("mass"))
        .def("clear_particles", &sph::SPHEngine::clear_particles)
        .def("step", &sph::SPHEngine::step, py::arg("dt") = 0.0f)
        .def("run_steps", &sph::SPHEngine::run_steps, py::arg("num_steps"),
             py::arg("adaptive_timestep") = true)
        .def("get_particles", &sph::SPHEngine::get_particles, py::return_value_policy::reference_internal)
        .def("get_parameters", &sph::SPHEngine::get_parameters)
        .def("get_current_time", &sph::SPHEngine::get_current_time)
        .def("get_step_count", &sph::SPHEngine::get_step_count)
        .def("set_parameters", &sph::SPHEngine::set_parameters)
        .def("set_gravity", &sph::SPHEngine::set_gravity)
        .def("set_viscosity", &sph::SPHEngine::set_viscosity)
        .def("set_smoothing_length", &sph::SPHEngine::set_smoothing_length)
        .def("set_boundaries", &sph::SPHEngine::set_boundaries)
        .def("set_kernel_type", &sph::SPHEngine::set_kernel_type)
        .def("get_kernel_type", &sph::SPHEngine::get_kernel_type)
        .def("get_performance_stats", &sph::SPHEngine::get_performance_stats,
             py::return_value_policy::copy)
        .def("reset_performance_stats", &sph::SPHEngine::reset_performance_stats)
        .def("compute_conservation_errors",
             [](sph::SPHEngine& e) {
                 float mass_error = 0.0f, energy_error = 0.0f;
                 e.compute_conservation_errors(mass_error, energy_error);
                 return py::make_tuple(mass_error, energy_error);
             })
        .def("get_total_mass", &sph::SPHEngine::get_total_mass)
        .def("get_total_energy", &sph::SPHEngine::get_total_energy)
        .def("get_conservation_sums", &sph::SPHEngine::get_conservation_sums)
        .def("validate_simulation", &sph::SPHEngine::validate_simulation)
        .def("is_initialized", &sph::SPHEngine::is_initialized)
        // the engine's getters, filled in place (the same values as the C++ getters)
        .def("get_positions", [](const sph::SPHEngine& e) {
            py::array_t<float> a({e.particle_count(), size_t(3)});
            e.copy_positions(a.mutable_data());
            return a;
        })
        .def("get_velocities", [](const sph::SPHEngine& e) {
            py::array_t<float> a({e.particle_count(), size_t(3)});
            e.copy_velocities(a.mutable_data());
            return a;
        })
        .def("get_densities", [](const sph::SPHEngine& e) {
            py::array_t<float> a(e.density_count());
            e.copy_densities(a.mutable_data());
            return a;
        })
        .def("get_pressures", [](const sph::SPHEngine& e) {
            py::array_t<float> a(e.density_count());
            e.copy_pressures(a.mutable_data());
            return a;
        });

    py::class_<sph::SpatialHash>(m, "SpatialHash")
        .def(py::init<float>(), py::arg("cell_size") = 0.02f)
        .def("build",
             [](sph::SpatialHash& h, py::array_t<float, py::array::c_style | py::array::forcecast> pos) {
                 if (pos.ndim() != 2 || pos.shape(1) != 3) throw std::invalid_argument("pos is (n, 3)");
                 std::vector<glm::vec3> v(static_cast<size_t>(pos.shape(0)));
                 for (size_t i = 0; i < v.size(); ++i)
                     v[i] = glm::vec3(pos.data()[3 * i], pos.data()[3 * i + 1], pos.data()[3 * i + 2]);
                 h.build(v);
             })
        .def("query", &sph::SpatialHash::query, py::arg("position"), py::arg("radius"))
        .def("query_squared", &sph::SpatialHash::query_squared, py::arg("position"),
             py::arg("radius_squared"))
        .def("get_cell_particles",
             [](const sph::SpatialHash& h, int x, int y, int z) -> py::object {
                 const std::vector<size_t>* v = h.get_cell_particles(x, y, z);
                 if (!v) return py::none();
                 return py::cast(*v);
             })
        .def("clear", &sph::SpatialHash::clear)
        .def("get_total_cells", &sph::SpatialHash::get_total_cells)
        .def("get_max_particles_per_cell", &sph::SpatialHash::get_max_particles_per_cell)
        .def("get_cell_size", &sph::SpatialHash::get_cell_size)
        .def("set_cell_size", &sph::SpatialHash::set_cell_size);

    m.def("create_fluid_block",
          [](const py::array_t<float, py::array::c_style | py::array::forcecast>& center,
             const py::array_t<float, py::array::c_style | py::array::forcecast>& size, float spacing,
             float mass) {
              return sph::create_fluid_block(vec3_from(center, "center"), vec3_from(size, "size"),
                                             spacing, mass);
          },
          py::arg("center"), py::arg("size"), py::arg("spacing"), py::arg("mass") = 1.0f);
    m.def("create_boundary_box",
          [](const py::array_t<float, py::array::c_style | py::array::forcecast>& center,
             const py::array_t<float, py::array::c_style | py::array::forcecast>& size, float spacing,
             float mass) {
              return sph::create_boundary_box(vec3_from(center, "center"), vec3_from(size, "size"),
                                              spacing, mass);
          },
          py::arg("center"), py::arg("size"), py::arg("spacing"), py::arg("mass") = 1.0f);

    // utils:: scene generators (src/sph_engine.cpp:450-552)
    m.def("create_dam_break_setup",
          [](const std::vector<float>& dam, const std::vector<float>& fluid, float spacing,
             const sph::SPHParameters& p) {
              if (dam.size() != 3 || fluid.size() != 3) throw std::invalid_argument("3D vectors expected");
              return sph::utils::create_dam_break_setup(glm::vec3(dam[0], dam[1], dam[2]),
                                                        glm::vec3(fluid[0], fluid[1], fluid[2]), spacing, p);
          },
          py::arg("dam_size"), py::arg("fluid_size"), py::arg("spacing"), py::arg("params"));
    m.def("create_fluid_drop_setup",
          [](const std::vector<float>& c, float radius, float spacing, const sph::SPHParameters& p) {
              if (c.size() != 3) throw std::invalid_argument("center must be a 3D vector");
              return sph::utils::create_fluid_drop_setup(glm::vec3(c[0], c[1], c[2]), radius, spacing, p);
          },
          py::arg("center"), py::arg("radius"), py::arg("spacing"), py::arg("params"));
    m.def("create_granular_flow_setup",
          [](const std::vector<float>& pile, const std::vector<float>& dom, float spacing,
             const sph::SPHParameters& p) {
              if (pile.size() != 3 || dom.size() != 3) throw std::invalid_argument("3D vectors expected");
              return sph::utils::create_granular_flow_setup(glm::vec3(pile[0], pile[1], pile[2]),
                                                            glm::vec3(dom[0], dom[1], dom[2]), spacing, p);
          },
          py::arg("pile_size"), py::arg("domain_size"), py::arg("spacing"), py::arg("params"));
    // flat record of a particle list: (n, 11) float32 = pos3 vel3 mass type color3
    m.def("particle_records", [](const std::vector<sph::Particle>& ps) {
        py::array_t<float> out({static_cast<py::ssize_t>(ps.size()), static_cast<py::ssize_t>(11)});
        auto r = out.mutable_unchecked<2>();
        for (size_t i = 0; i < ps.size(); ++i) {
            const sph::Particle& p = ps[i];
            const float v[11] = {p.position.x, p.position.y, p.position.z, p.velocity.x, p.velocity.y,
                                 p.velocity.z, p.mass, static_cast<float>(static_cast<int>(p.type)),
                                 p.color.x, p.color.y, p.color.z};
            for (int k = 0; k < 11; ++k) r(i, k) = v[k];
        }
        return out;
    });

    m.attr("__version__") = "1.0.0";
}
