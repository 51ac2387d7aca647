"""GPU step parity, through the C ABI, against the oracle.

The oracle here is the C restatement of the reference step, itself pinned bit for bit to
the reference's own code by tests/test_oracle.py and to the reference-generated fixtures
in tests/golden/.  In SPHX_MODE_EXACT the GPU must reproduce every field bit for bit:
neighbour lists in the reference's order, density, pressure, acceleration, and after a
step position, velocity and time (NaN compares equal to NaN).
"""
import numpy as np
import pytest

import sph_oracle as O
import sphx
import sphx_inputs as I
from conftest import GOLDEN_CASES, golden_case

pytestmark = pytest.mark.gpu


def make_ctx(n, params, pos, vel, mass, **kw):
    ctx = sphx.Context(max(n, 1), **kw)
    ctx.set_params(params)
    ctx.upload(pos, vel, mass)
    return ctx


def assert_bits(a, b, name):
    assert O.bits_equal(a, b), O.mismatch_report(a, b, name)


# ---- against the reference-generated fixtures ----------------------------------------

@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gpu_neighbour_lists_match_reference_fixture(built, golden, case):
    g = golden_case(golden, case)
    ctx = make_ctx(g["pos"].shape[0], g["params"], g["pos"], g["vel"], g["mass"])
    counts, idx = ctx.pairs()
    assert np.array_equal(counts, g["counts"])
    assert np.array_equal(idx, g["idx"].astype(np.int64))  # same order


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gpu_fields_match_reference_fixture(built, golden, case):
    g = golden_case(golden, case)
    ctx = make_ctx(g["pos"].shape[0], g["params"], g["pos"], g["vel"], g["mass"])
    ctx.eval()
    out = ctx.download()
    assert_bits(out["rho"], g["rho"], "rho")
    assert_bits(out["pressure"], g["pressure"], "P")
    assert_bits(out["acc"], g["acc"], "acc")
    assert_bits(out["pos"], g["pos"], "pos unchanged by eval")


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gpu_trajectory_matches_reference_fixture(built, golden, case):
    g = golden_case(golden, case)
    ctx = make_ctx(g["pos"].shape[0], g["params"], g["pos"], g["vel"], g["mass"])
    for s, dt in enumerate(g["dts"]):
        ctx.step(float(dt))
        out = ctx.download(acc=False)
        assert_bits(out["pos"], g["traj_pos"][s], f"pos@{s}")
        assert_bits(out["vel"], g["traj_vel"][s], f"vel@{s}")
        assert_bits(out["rho"], g["traj_rho"][s], f"rho@{s}")
        assert_bits(out["pressure"], g["traj_pressure"][s], f"P@{s}")
        t, _ = ctx.time()
        assert np.float32(t) == g["traj_time"][s]


# ---- against the oracle on the dam-break workloads ------------------------------------

def test_gpu_10k_dam_break_trajectory_fixed_and_adaptive(port):
    w = I.config0()
    for dt in (1e-3, 0.0):
        ctx = make_ctx(w.n, w.params, w.pos, w.vel, w.mass)
        e = O.Engine(port, w.n)
        e.initialize(w.params)
        e.add(w.pos, w.vel, w.mass)
        for s in range(12):
            ctx.step(dt)
            e.step(dt)
            out = ctx.download()
            ref = e.get()
            for k in ("pos", "vel", "rho", "pressure", "acc"):
                assert_bits(out[k], ref[k], f"{k}@{s} dt={dt}")
            t, last = ctx.time()
            assert t == e.time() and last == e.last_dt()
        st = ctx.stats()
        d = e.diag()
        assert st["max_neighbors"] == d[4]
        assert st["total_neighbor_queries"] == d[5]


def test_gpu_neighbour_lists_100k(port):
    w = I.scaled_dam_break(100_000, seed=5)
    ctx = make_ctx(w.n, w.params, w.pos, w.vel, w.mass)
    c_gpu, i_gpu = ctx.pairs()
    c_ref, i_ref = port.query(w.pos, 0.04)
    assert np.array_equal(c_gpu, c_ref)
    assert np.array_equal(i_gpu, i_ref)


def test_gpu_1M_dam_break_fresh_step_bit_exact(port):
    """Configuration 1 (1,000,000 particles): one field evaluation and one step from the
    initial state, every field bit-identical to the oracle."""
    w = I.config1()
    ctx = make_ctx(w.n, w.params, w.pos, w.vel, w.mass)
    ctx.eval()
    out = ctx.download()
    rho, P, acc = port.fields(w.pos, w.vel, w.mass, w.params)
    assert_bits(out["rho"], rho, "rho")
    assert_bits(out["pressure"], P, "P")
    assert_bits(out["acc"], acc, "acc")
    e = O.Engine(port, w.n)
    e.initialize(w.params)
    e.add(w.pos, w.vel, w.mass)
    e.step(w.dt)
    ctx.step(w.dt)
    out = ctx.download(acc=False)
    ref = e.get()
    for k in ("pos", "vel", "rho", "pressure"):
        assert_bits(out[k], ref[k], k)


def test_gpu_density_error_against_fp64(port):
    """Stated accuracy: density relative error <= 1e-5 against the FP64 re-evaluation."""
    w = I.scaled_dam_break(200_000, seed=3)
    ctx = make_ctx(w.n, w.params, w.pos, w.vel, w.mass)
    ctx.eval()
    rho = ctx.download()["rho"].astype(np.float64)
    rho64, _, _ = port.fields_f64(w.pos, w.vel, w.mass, w.params)
    rel = np.abs(rho - rho64) / np.abs(rho64)
    assert rel.max() <= 1e-5, rel.max()


def test_gpu_fresh_state_restore(port):
    w = I.config0()
    ctx = make_ctx(w.n, w.params, w.pos, w.vel, w.mass)
    ctx.snapshot()
    ctx.step(w.dt)
    a = ctx.download()
    for _ in range(3):
        ctx.restore()
        ctx.step(w.dt)
        b = ctx.download()
        for k in ("pos", "vel", "rho"):
            assert_bits(a[k], b[k], k)


# ---- edge cases ----------------------------------------------------------------------

def test_gpu_single_particle_and_empty(port):
    prm = I.params16()
    ctx = sphx.Context(8)
    ctx.set_params(prm)
    ctx.step(1e-3)  # empty: no-op
    assert ctx.time()[0] == 0.0
    pos = np.array([[0.1, 0.2, 0.3]], np.float32)
    ctx.upload(pos, None, np.array([1e-3], np.float32))
    ctx.step(1e-3)
    e = O.Engine(port, 8)
    e.initialize(prm)
    e.add(pos, None, np.array([1e-3], np.float32))
    e.step(1e-3)
    out, ref = ctx.download(), e.get()
    for k in ("pos", "vel", "rho", "pressure"):
        assert_bits(out[k], ref[k], k)


def test_gpu_all_particles_in_one_cell_and_coincident(port):
    rng = np.random.default_rng(4)
    pos = (0.5 + rng.random((700, 3)) * 0.03).astype(np.float32)
    pos[100:140] = pos[99]  # 41 coincident particles
    vel = (rng.standard_normal((700, 3)) * 0.1).astype(np.float32)
    mass = np.full(700, 1e-3, np.float32)
    prm = I.params16(xmin=0, xmax=1, ymin=0, ymax=1, zmin=0, zmax=1)
    ctx = make_ctx(700, prm, pos, vel, mass)
    c1, i1 = ctx.pairs()
    c2, i2 = port.query(pos, 0.04)
    assert np.array_equal(c1, c2) and np.array_equal(i1, i2)
    ctx.eval()
    out = ctx.download()
    for a, b, k in zip((out["rho"], out["pressure"], out["acc"]),
                       port.fields(pos, vel, mass, prm), ("rho", "P", "acc")):
        assert_bits(a, b, k)


def test_gpu_tiny_coordinates_near_the_origin(port):
    """Particles within 1e-36 of the origin (normal and subnormal coordinates) beside
    particles at the origin, ordinary ones, and ones whose x alone is tiny: pair terms
    with zero distances and with gradient components below 2^-100, where the passes leave
    the untested divisions by h for the range-tested ones; fields and one step stay
    bit-identical to the oracle."""
    rng = np.random.default_rng(9)
    tiny = (rng.integers(-6, 7, size=(300, 3)) * 1e-37).astype(np.float32)
    sub = (rng.integers(-50, 51, size=(100, 3)) * 1e-44).astype(np.float32)
    zero = np.zeros((20, 3), np.float32)
    near = (0.01 + rng.random((200, 3)) * 0.02).astype(np.float32)
    # x tiny or 0 while y, z are ordinary: |r| is ordinary, the x component of r / |r| tiny
    axis = (0.01 + rng.random((200, 3)) * 0.02).astype(np.float32)
    axis[:, 0] = (rng.integers(-3, 4, size=200) * 1e-38).astype(np.float32)
    pos = np.concatenate([tiny, sub, zero, near, axis])
    assert (np.abs(sub[sub != 0]) < np.finfo(np.float32).tiny).all()
    vel = (rng.standard_normal(pos.shape) * 0.1).astype(np.float32)
    mass = np.full(len(pos), 1e-3, np.float32)
    prm = I.params16(xmin=-1, xmax=1, ymin=-1, ymax=1, zmin=-1, zmax=1)
    ctx = make_ctx(len(pos), prm, pos, vel, mass)
    ctx.eval()
    out = ctx.download()
    for a, b, k in zip((out["rho"], out["pressure"], out["acc"]),
                       port.fields(pos, vel, mass, prm), ("rho", "P", "acc")):
        assert_bits(a, b, k)
    ctx.step(1e-3)
    e = O.Engine(port, len(pos))
    e.initialize(prm)
    e.add(pos, vel, mass)
    e.step(1e-3)
    out, ref = ctx.download(), e.get()
    for k in ("pos", "vel", "rho", "pressure", "acc"):
        assert_bits(out[k], ref[k], k)


def test_gpu_crowded_cell_every_pair_a_neighbour(port):
    """640 particles inside a 0.015 cube (every pair within r = 0.04, full tiles): the
    force pass sums each lane's terms directly, chunk by chunk; one step stays
    bit-identical to the oracle."""
    rng = np.random.default_rng(12)
    pos = (0.5 + rng.random((640, 3)) * 0.015).astype(np.float32)
    vel = (rng.standard_normal((640, 3)) * 0.1).astype(np.float32)
    mass = np.full(640, 1e-3, np.float32)
    prm = I.params16(xmin=0, xmax=1, ymin=0, ymax=1, zmin=0, zmax=1)
    ctx = make_ctx(640, prm, pos, vel, mass)
    ctx.step(1e-4)
    e = O.Engine(port, 640)
    e.initialize(prm)
    e.add(pos, vel, mass)
    e.step(1e-4)
    out, ref = ctx.download(), e.get()
    for k in ("pos", "vel", "rho", "pressure", "acc"):
        assert_bits(out[k], ref[k], k)


def test_gpu_capacity_and_parameter_errors():
    ctx = sphx.Context(4)
    with pytest.raises(sphx.SphxError) as ei:
        ctx.upload(np.zeros((5, 3), np.float32), None, np.ones(5, np.float32))
    assert ei.value.code == -5
    with pytest.raises(sphx.SphxError) as ei:
        ctx.set_params(I.params16(neighbor_search_radius=0.0))
    assert ei.value.code == -1
    ctx.upload(np.zeros((2, 3), np.float32), None, np.ones(2, np.float32))
    with pytest.raises(sphx.SphxError) as ei:
        ctx.step(1e-3)  # no parameters yet
    assert ei.value.code == -6


@pytest.mark.parametrize("max_cells", [125, 1000, 0])
def test_gpu_huge_box_folds_the_grid(port, max_cells):
    """Particles spread over a box far larger than the cell grid: the grid folds, and
    lists, order and fields stay bit-identical (cells that fold together are far apart)."""
    rng = np.random.default_rng(8)
    clusters = [np.array(c, np.float32) for c in ((0, 0, 0), (10, 10, 10), (3.3, -7.1, 0.2),
                                                   (250.0, 0.0, -40.0))]
    pos = np.concatenate([c + rng.random((300, 3)).astype(np.float32) * 0.12 for c in clusters])
    n = pos.shape[0]
    vel = (rng.standard_normal((n, 3)) * 0.1).astype(np.float32)
    mass = np.full(n, 1e-3, np.float32)
    prm = I.params16(xmin=-100, xmax=300, ymin=-100, ymax=100, zmin=-100, zmax=100)
    ctx = make_ctx(n, prm, pos, vel, mass, max_grid_cells=max_cells)
    c1, i1 = ctx.pairs()
    c2, i2 = port.query(pos, 0.04)
    assert np.array_equal(c1, c2) and np.array_equal(i1, i2)
    ctx.eval()
    out = ctx.download()
    for a, b, k in zip((out["rho"], out["pressure"], out["acc"]),
                       port.fields(pos, vel, mass, prm), ("rho", "P", "acc")):
        assert_bits(a, b, k)
    st = ctx.stats()
    if max_cells:
        assert st["grid_cells"] <= max(max_cells, 125)


@pytest.mark.parametrize("tile", [7, 16, 24])
def test_gpu_tile_sizes_keep_every_field_bit_exact(port, tile):
    """Tiles of fewer particles per warp work item (a tuning choice) change only how the
    work is split: one step stays bit-identical to the oracle."""
    w = I.scaled_dam_break(60_000, seed=17)
    ctx = make_ctx(w.n, w.params, w.pos, w.vel, w.mass, tile_particles=tile)
    assert ctx.tuning()["tile_particles"] == tile
    ctx.step(w.dt)
    e = O.Engine(port, w.n)
    e.initialize(w.params)
    e.add(w.pos, w.vel, w.mass)
    e.step(w.dt)
    out, ref = ctx.download(), e.get()
    for k in ("pos", "vel", "rho", "pressure", "acc"):
        assert_bits(out[k], ref[k], k)


@pytest.mark.parametrize("case", ["lattice_60k", "crowded", "edge"])
def test_gpu_bulk_copy_staging_keeps_every_field_bit_exact(port, golden, case):
    """The force pass's bulk-copy staging (cp.async.bulk into double buffers, a tuning
    choice) changes only how candidates reach shared memory: one step bit-identical to the
    oracle on the lattice, a crowded cell and the reference's edge fixture."""
    if case == "lattice_60k":
        w = I.scaled_dam_break(60_000, seed=17)
        pos, vel, mass, prm, dt = w.pos, w.vel, w.mass, w.params, w.dt
    elif case == "crowded":
        rng = np.random.default_rng(12)
        pos = (0.5 + rng.random((640, 3)) * 0.015).astype(np.float32)
        vel = (rng.standard_normal((640, 3)) * 0.1).astype(np.float32)
        mass = np.full(640, 1e-3, np.float32)
        prm, dt = I.params16(xmin=0, xmax=1, ymin=0, ymax=1, zmin=0, zmax=1), 1e-4
    else:
        g = golden_case(golden, "edge")
        pos, vel, mass, prm, dt = g["pos"], g["vel"], g["mass"], g["params"], 1e-3
    n = pos.shape[0]
    ctx = make_ctx(n, prm, pos, vel, mass, bulk_copy=True)
    assert ctx.tuning()["bulk_copy"] == 1
    ctx.step(dt)
    e = O.Engine(port, n)
    e.initialize(prm)
    e.add(pos, vel, mass)
    e.step(dt)
    out, ref = ctx.download(), e.get()
    for k in ("pos", "vel", "rho", "pressure", "acc"):
        assert_bits(out[k], ref[k], k)
