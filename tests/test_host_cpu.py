"""The C++ drop-in engine and its pybind11 module `sph`, host side (no GPU needed).

The module must expose the reference's Python names (python/bindings.cpp:8-166) and its
scene generators must reproduce the reference's initial conditions bit for bit (pinned
by the SHA-256 of the reference's own initialize_* particle records in tests/golden/).
"""
import hashlib
import sys

import numpy as np
import pytest

from conftest import PKG

sys.path.insert(0, str(PKG / "lib"))


@pytest.fixture(scope="module")
def sph(built):
    import sphx_build

    sphx_build.build_host()
    if sphx_build.build_pymodule() is None:
        pytest.skip("Python headers or pybind11 headers missing on this machine")
    import sph as mod

    return mod


def test_module_surface_matches_reference_bindings(sph):
    for name in ("SPHParameters", "ParticleType", "Particle", "ParticleSystem",
                 "PerformanceStats", "Simulator", "create_fluid_block", "create_boundary_box"):
        assert hasattr(sph, name), name
    for meth in ("initialize", "initialize_dam_break", "initialize_fluid_drop",
                 "initialize_granular_flow", "add_particles", "clear_particles", "step",
                 "run_steps", "get_particles", "get_parameters", "get_current_time",
                 "get_step_count", "set_parameters", "set_gravity", "set_viscosity",
                 "set_smoothing_length", "set_boundaries", "get_performance_stats",
                 "reset_performance_stats", "compute_conservation_errors", "get_total_mass",
                 "get_total_energy", "validate_simulation", "is_initialized", "get_positions",
                 "get_velocities", "get_densities", "get_pressures"):
        assert hasattr(sph.Simulator, meth), meth
    assert sph.__version__ == "1.0.0"


def test_parameters_defaults(sph):
    p = sph.SPHParameters()
    vals = (p.rest_density, p.gas_constant, p.viscosity, p.smoothing_length, p.particle_mass,
            p.timestep, p.gravity, p.damping, p.CFL_factor, p.neighbor_search_radius)
    want = (1000.0, 2000.0, 0.001, 0.02, 0.001, 0.001, -9.81, 0.99, 0.4, 0.04)
    assert np.allclose(vals, want)
    assert p.bounds == pytest.approx((-1, 1, -1, 1, -1, 1))


def test_particle_record(sph):
    q = sph.Particle([0.1, 0.2, 0.3], 2.0, sph.ParticleType.BOUNDARY)
    assert (q.position.x, q.position.y, q.position.z) == pytest.approx((0.1, 0.2, 0.3))
    assert q.mass == 2.0 and q.type == sph.ParticleType.BOUNDARY and q.id == -1
    assert q.temperature == pytest.approx(293.15) and q.viscosity == pytest.approx(0.001)
    d = sph.Particle()
    assert d.mass == 1.0 and d.type == sph.ParticleType.FLUID


def test_create_fluid_block_shape_and_rejects_bad_vectors(sph):
    ps = sph.create_fluid_block([0, 0, 0], [0.1, 0.05, 0.02], 0.01, 1e-3)
    assert len(ps) == 10 * 5 * 2
    with pytest.raises(ValueError):
        sph.create_fluid_block([0, 0], [0.1, 0.1, 0.1], 0.01)


@pytest.mark.parametrize("scene", ["dam_break", "fluid_drop", "granular_flow"])
def test_scene_generators_match_reference(sph, golden, scene):
    p = sph.SPHParameters()
    if scene == "dam_break":
        ps = sph.create_dam_break_setup([0.4, 0.6, 0.8], [0.2, 0.4, 0.8], 0.01, p)
    elif scene == "fluid_drop":
        ps = sph.create_fluid_drop_setup([0.0, 0.5, 0.0], 0.1, 0.008, p)
    else:
        ps = sph.create_granular_flow_setup([0.3, 0.4, 0.8], [1.0, 1.0, 1.0], 0.012, p)
    rec = np.ascontiguousarray(sph.particle_records(ps), np.float32)
    assert rec.shape[0] == int(golden[f"scene/{scene}/n"])
    assert np.array_equal(rec[:8].view(np.uint32), golden[f"scene/{scene}/first"].view(np.uint32))
    digest = np.frombuffer(hashlib.sha256(rec.tobytes()).digest(), np.uint8)
    assert np.array_equal(digest, golden[f"scene/{scene}/sha256"])


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("h", [0.02, 0.0137])
def test_kernel_objects_match_reference(sph, golden, kind, h):
    """create_kernel(type, h)->W / gradW / laplacianW give the reference's bits
    (fixture from the reference's own kernel classes, src/kernels.cpp:140-236)."""
    import sph_oracle as O

    key = f"kernel/k{kind}_h{h}"
    r = golden[key + "/r"]
    k = sph.create_kernel(sph.KernelType(kind), h)
    w = np.array([k.W(sph.vec3(*map(float, v))) for v in r], np.float32)
    g = np.array([[c.x, c.y, c.z] for c in (k.gradW(sph.vec3(*map(float, v))) for v in r)],
                 np.float32)
    lap = np.array([k.laplacianW(sph.vec3(*map(float, v))) for v in r], np.float32)
    assert O.bits_equal(w, golden[key + "/W"]), O.mismatch_report(w, golden[key + "/W"], "W")
    assert O.bits_equal(g, golden[key + "/gradW"]), O.mismatch_report(g, golden[key + "/gradW"], "gradW")
    assert O.bits_equal(lap, golden[key + "/laplacianW"]), O.mismatch_report(
        lap, golden[key + "/laplacianW"], "laplacianW")
    assert k.get_support_radius() == np.float32(2.0) * np.float32(h)


def test_kernel_factory_rejects_unknown_type_and_engine_default(sph):
    with pytest.raises((ValueError, TypeError)):
        sph.create_kernel(sph.KernelType(7), 0.02)
    assert int(sph.KernelType.WENDLAND_C2) == 1 and int(sph.KernelType.GAUSSIAN) == 2


def test_camera_matrices_follow_the_gl_conventions(built):
    """sphx_camera_matrices (host code): look-at of the reference's Camera and an OpenGL
    perspective (near 0.1, far 100), checked against the textbook formulas in FP64."""
    import sphx

    for pos, yaw, pitch, fov, aspect in [((0, 0, 3), -90, 0, 45, 16 / 9),
                                         ((1.8, 1.2, 1.6), -135, -25, 35, 4 / 3)]:
        view, proj = sphx.camera_matrices(pos, yaw, pitch, fov, aspect)
        V = view.reshape(4, 4).T.astype(np.float64)  # column-major -> row-major
        Pm = proj.reshape(4, 4).T.astype(np.float64)
        y, p = np.radians(yaw), np.radians(pitch)
        f = np.array([np.cos(y) * np.cos(p), np.sin(p), np.sin(y) * np.cos(p)])
        f /= np.linalg.norm(f)
        s = np.cross(f, [0, 1, 0])
        s /= np.linalg.norm(s)
        u = np.cross(s, f)
        e = np.array(pos, np.float64)
        want_v = np.eye(4)
        want_v[0, :3], want_v[1, :3], want_v[2, :3] = s, u, -f
        want_v[:3, 3] = [-s @ e, -u @ e, f @ e]
        assert np.abs(V - want_v).max() < 1e-5
        t = np.tan(np.radians(fov) / 2)
        want_p = np.zeros((4, 4))
        want_p[0, 0], want_p[1, 1] = 1 / (aspect * t), 1 / t
        want_p[2, 2], want_p[2, 3], want_p[3, 2] = -100.1 / 99.9, -2 * 100 * 0.1 / 99.9, -1
        assert np.abs(Pm - want_p).max() < 1e-5 * np.abs(want_p).max()
        # the eye maps to the view-space origin, a point ahead of it to -z
        assert np.abs(V @ np.append(e, 1))[:3].max() < 1e-5
        assert (V @ np.append(e + f, 1))[2] == pytest.approx(-1.0, abs=1e-5)
