"""The drop-in engine (C++ sph::SPHEngine through the pybind11 module `sph`) and the
GPU spatial hash, against the oracle.

Same results as the reference engine, bit for bit, through the reference's own API:
initialise, add particles, step (fixed and adaptive dt), read positions, velocities,
capacity-length densities/pressures, particle records, time, statistics; parameter
setters with the reference's rules; SpatialHash lists in the reference's order.
"""
import sys

import numpy as np
import pytest

import sph_oracle as O
import sphx
import sphx_inputs as I
from conftest import PKG

pytestmark = pytest.mark.gpu
sys.path.insert(0, str(PKG / "lib"))


@pytest.fixture(scope="module")
def sph(built):
    import sphx_build

    if sphx_build.build_pymodule() is None:
        pytest.skip("Python headers or pybind11 headers missing on this machine")
    import sph as mod

    return mod


def params_obj(sph, p16):
    p = sph.SPHParameters()
    (p.rest_density, p.gas_constant, p.viscosity, p.smoothing_length, p.particle_mass,
     p.timestep, p.gravity, p.damping, p.CFL_factor) = [float(x) for x in p16[:9]]
    p.bounds = [float(x) for x in p16[9:15]]
    p.neighbor_search_radius = float(p16[15])
    return p


def bits(a, b, name):
    assert O.bits_equal(a, b), O.mismatch_report(a, b, name)


@pytest.mark.parametrize("dt", [1e-3, 0.0])
def test_simulator_matches_oracle_engine(sph, port, dt):
    w = I.config0()
    cap = w.n + 500
    sim = sph.Simulator(cap)
    sim.initialize(params_obj(sph, w.params))
    sim.add_particles_array(w.pos, w.vel, w.mass)
    e = O.Engine(port, cap)
    e.initialize(w.params)
    e.add(w.pos, w.vel, w.mass)
    for s in range(6):
        sim.step(dt)
        e.step(dt)
        ref = e.get()
        bits(sim.get_positions(), ref["pos"], f"pos@{s}")
        bits(sim.get_velocities(), ref["vel"], f"vel@{s}")
        dens = sim.get_densities()
        assert dens.shape == (cap,)  # capacity-length, like the reference
        bits(dens, ref["rho_cap"], f"rho@{s}")
        bits(sim.get_pressures(), ref["pressure_cap"], f"P@{s}")
        assert sim.get_current_time() == e.time()
        assert sim.get_step_count() == s + 1
    d = e.diag()
    assert sim.get_total_mass() == np.float32(d[0])
    assert sim.get_total_energy() == np.float32(d[1])
    me, ee = sim.compute_conservation_errors()
    assert me == np.float32(d[2]) and ee == 0.0
    st = sim.get_performance_stats()
    assert st.max_neighbors == d[4] and st.total_neighbor_queries == d[5]
    assert st.total_time > 0 and st.force_computation_time > 0
    ps = sim.get_particles()
    assert ps.size() == w.n and ps.capacity() == cap
    rec = ps[17]
    assert rec.density == ref["rho"][17] and rec.pressure == ref["pressure"][17]
    assert (rec.acceleration.x, rec.acceleration.y, rec.acceleration.z) == (0.0, 0.0, 0.0)


def test_simulator_scene_and_host_changes_between_steps(sph, port):
    sim = sph.Simulator(200_000)
    sim.initialize_fluid_drop()  # default parameters (initialize(SPHParameters{}))
    assert sim.is_initialized()
    ps = sim.get_particles()
    pos0 = ps.get_positions().copy()
    n0 = ps.size()
    prm = I.params16()
    e = O.Engine(port, 200_000)
    e.initialize(prm)
    e.add(pos0, None, np.full(n0, 1e-3, np.float32))
    for _ in range(2):
        sim.step()
        e.step(0.0)
    # adding particles after a step: the host mirror syncs, the device is re-uploaded
    extra = I.lattice(4, 4, 4, seed=3) + np.float32(0.3)
    sim.add_particles_array(extra, None, np.full(64, 1e-3, np.float32))
    e.add(extra, None, np.full(64, 1e-3, np.float32))
    sim.step(5e-4)
    e.step(5e-4)
    ref = e.get()
    bits(sim.get_positions(), ref["pos"], "pos")
    bits(sim.get_densities()[: n0 + 64], ref["rho"], "rho")
    assert sim.get_current_time() == e.time()
    sim.clear_particles()
    assert sim.get_current_time() == 0.0 and sim.get_step_count() == 0
    assert sim.get_particles().size() == 0
    sim.step(1e-3)  # empty: no-op
    assert sim.get_step_count() == 0


def test_parameter_rules(sph):
    sim = sph.Simulator(100)
    p = sph.SPHParameters()
    p.smoothing_length = 0.03
    p.neighbor_search_radius = 0.05
    sim.initialize(p)  # initialize keeps the given radius
    assert sim.get_parameters().neighbor_search_radius == pytest.approx(0.05)
    sim.set_parameters(p)  # set_parameters forces radius = 2h
    assert sim.get_parameters().neighbor_search_radius == pytest.approx(0.06)
    sim.set_smoothing_length(0.01)
    assert sim.get_parameters().neighbor_search_radius == pytest.approx(0.02)
    sim.set_gravity(-1.0)
    sim.set_viscosity(0.5)
    sim.set_boundaries(0, 1, 0, 2, 0, 3)
    q = sim.get_parameters()
    assert q.gravity == -1.0 and q.viscosity == 0.5 and q.bounds == pytest.approx((0, 1, 0, 2, 0, 3))
    assert sim.get_densities().shape == (100,)


def test_capacity_drop(sph, capfd):
    sim = sph.Simulator(3)
    sim.initialize(sph.SPHParameters())
    sim.add_particles([sph.Particle([0.1 * k, 0, 0], 1e-3) for k in range(5)])
    assert sim.get_particles().size() == 3
    assert "capacity exceeded" in capfd.readouterr().err


@pytest.mark.parametrize("cell", [0.04, 0.02, 0.05])
def test_spatial_hash_matches_reference_order(sph, port, cell):
    w = I.scaled_dam_break(30_000, seed=6)
    h = sph.SpatialHash(cell)
    h.build(w.pos)
    r = np.float32(0.04)
    r2 = r * r  # float32, as SPHEngine passes radius * radius
    c2, i2 = port.query(w.pos, float(r), cell_size=cell)  # every particle's list
    for i in (0, 17, 12345, w.n - 1):
        got = np.array(h.query_squared(w.pos[i], r2), np.int64)
        start = int(np.sum(c2[:i]))
        assert np.array_equal(got, i2[start:start + c2[i]])
    assert h.get_total_cells() > 0
    assert h.get_max_particles_per_cell() >= 1
    inv = np.float32(1.0) / np.float32(cell)
    c = np.floor(w.pos[5] * inv).astype(int)
    members = h.get_cell_particles(int(c[0]), int(c[1]), int(c[2]))
    assert 5 in members and members == sorted(members)


def test_grid_abi_batched_queries(port):
    w = I.scaled_dam_break(20_000, seed=9)
    g = sphx.Grid(w.n)
    g.build(w.pos, 0.02)  # cells of half the radius: the stencil is 7 cells wide
    counts, idx = g.query(w.pos, np.float32(0.04) * np.float32(0.04))
    c2, i2 = port.query(w.pos, 0.04, cell_size=0.02)
    assert np.array_equal(counts, c2) and np.array_equal(idx, i2)
    # query points that are not particles, including a NaN one
    q = np.array([[0.5, 0.5, 0.5], [np.nan, 0.1, 0.1], [5.0, 5.0, 5.0]], np.float32)
    counts, idx = g.query(q, np.float32(0.04) * np.float32(0.04))
    assert counts[1] == 0 and counts[2] == 0
    cells, mx = g.info()
    assert cells > 0 and mx >= 1


def test_simulator_kernel_type_matches_oracle_engine(sph, port):
    """set_kernel_type(WENDLAND_C2): the engine's step equals the oracle engine stepping
    with create_kernel(WENDLAND_C2); the choice survives set_smoothing_length."""
    w = I.config0()
    sim = sph.Simulator(w.n)
    sim.initialize(params_obj(sph, w.params))
    sim.set_kernel_type(sph.KernelType.WENDLAND_C2)
    assert sim.get_kernel_type() == sph.KernelType.WENDLAND_C2
    sim.add_particles_array(w.pos, w.vel, w.mass)
    e = O.Engine(port, w.n)
    e.set_kernel(1)
    e.initialize(w.params)
    e.add(w.pos, w.vel, w.mass)
    for s, dt in enumerate([1e-3, 0.0, 1e-3]):
        sim.step(dt)
        e.step(dt)
        ref = e.get()
        bits(sim.get_positions(), ref["pos"], f"pos@{s}")
        bits(sim.get_densities(), ref["rho_cap"], f"rho@{s}")
    sim.set_smoothing_length(0.02)
    assert sim.get_kernel_type() == sph.KernelType.WENDLAND_C2
