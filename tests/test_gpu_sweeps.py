"""The precision mode's tile sweeps on the paths the dam break does not take, against the
FP64 evaluation of the reference's step formulas (the oracle's fields_f64: the same
neighbour sets, |r|^2 <= r_search^2, and the reference's W / gradW / laplacianW).

Stated accuracy, as for the precision mode elsewhere: density relative error <= 1e-5;
acceleration error per component <= 1e-4 of the sum of the magnitudes of its terms.

* a search radius below the support 2h: the sweep masks every term by the neighbour test
  (the max form alone would keep pairs between r_search and 2h).  The kernel does not
  vanish at such a cutoff, so a pair within rounding of r_search changes a density by
  O(W(r)) depending on which side of the test it falls: the case uses an unjittered lattice
  with r_search between two lattice distances, where no pair is near the cutoff;
* a search radius above 2h: pairs between 2h and r_search are neighbours whose terms are 0;
* a non-finite velocity: the chunks that stage it take the masked sweep, so it reaches
  exactly the particle's neighbours (as in the reference) and no other particle of the
  tiles that see it;
* collapsed cells (more than 128 particles, kept in insertion order, tiles spanning many
  cells of a column), thousands of neighbours per particle.  The sparse particles around
  the cluster, some with a single neighbour near q = 2, are held to 1e-3 instead: there
  (2 - q)^2 carries the rounding of q relative to 2 - q, in every float evaluation (the
  reference's too), and one term is all of the sum;
* the tile sizes the autotuner tries;
* a grid folded on every axis (a box far larger than the cell grid): cells that fold
  together are far apart, so a column tile can hold particles of clusters far apart (a
  spread tile, swept with each lane's own cell as its frame), and its rows pick up far
  candidates from the folded cells.  The isolated particles of this case and of the
  collapsed one (a single neighbour: the particle itself) must get exactly no force.
"""
import numpy as np
import pytest

import sphx
import sphx_inputs as I

pytestmark = pytest.mark.gpu

RHO_TOL, ACC_TAU = 1e-5, 1e-4


def precise_fields(pos, vel, mass, prm, tile=0, stats=None):
    ctx = sphx.Context(max(pos.shape[0], 1), mode=sphx.MODE_PRECISE, tile_particles=tile)
    ctx.set_params(prm)
    ctx.upload(pos, vel, mass)
    ctx.eval()
    out = ctx.download(pos=False, vel=False)
    if stats is not None:
        stats.update(ctx.stats())
    ctx.close()
    return out


def check_against_fp64(port, pos, vel, mass, prm, out, finite_only=False, sel=None,
                       acc_tau=ACC_TAU):
    rho64, _, acc64, scale = port.fields_f64(pos, vel, mass, prm, want_scale=True)
    ok = np.isfinite(acc64).all(axis=1) if finite_only else np.ones(len(rho64), bool)
    if sel is not None:
        ok &= sel
    rel = np.abs(out["rho"][ok] - rho64[ok]) / rho64[ok]
    assert rel.max() <= RHO_TOL, rel.max()
    err = np.abs(out["acc"][ok] - acc64[ok]) / np.maximum(scale[ok], 1e-30)
    assert err.max() <= acc_tau, err.max()
    return rho64, acc64


def plain_lattice(side, spacing=0.01, origin=0.1):
    k = np.arange(side, dtype=np.float32) * np.float32(spacing) + np.float32(origin)
    gx, gy, gz = np.meshgrid(k, k, k, indexing="ij")
    pos = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1).astype(np.float32)
    rng = np.random.default_rng(side)
    vel = (0.1 * rng.standard_normal(pos.shape)).astype(np.float32)
    return pos, vel, np.full(len(pos), 1e-3, np.float32)


# lattice distances are 0.01 sqrt(k): 0.0308 lies between sqrt(9) and sqrt(10), 0.0495
# between sqrt(24) and sqrt(25)
@pytest.mark.parametrize("radius", [0.0308, 0.0495])
def test_search_radius_other_than_2h(port, radius):
    pos, vel, mass = plain_lattice(40)
    prm = I.params16(neighbor_search_radius=radius)
    out = precise_fields(pos, vel, mass, prm)
    check_against_fp64(port, pos, vel, mass, prm, out)


def test_nonfinite_velocity_reaches_only_its_neighbours(port):
    w = I.scaled_dam_break(60_000, seed=22)
    vel = w.vel.copy()
    k = len(vel) // 2 + 17  # a particle inside the block
    vel[k] = np.float32("nan")
    out = precise_fields(w.pos, vel, w.mass, w.params)
    rho64, acc64 = check_against_fp64(port, w.pos, vel, w.mass, w.params, out, finite_only=True)
    bad_gpu = ~np.isfinite(out["acc"]).all(axis=1)
    bad_64 = ~np.isfinite(acc64).all(axis=1)
    assert bad_64.sum() > 10  # the particle's neighbours
    assert np.array_equal(bad_gpu, bad_64)
    assert np.isfinite(out["rho"]).all()


def test_collapsed_cells_thousands_of_neighbours(port):
    rng = np.random.default_rng(23)
    n = 12_000
    pos = np.empty((n, 3), np.float32)
    pos[: n - 2000] = 0.5 + 0.03 * rng.random((n - 2000, 3), dtype=np.float32)  # a few cells
    pos[n - 2000:] = 0.2 + 0.6 * rng.random((2000, 3), dtype=np.float32)  # sparse rest
    vel = (0.1 * rng.standard_normal((n, 3))).astype(np.float32)
    mass = np.full(n, 1e-3, np.float32)
    prm = I.params16()
    out = precise_fields(pos, vel, mass, prm)
    counts, _ = port.query(pos, 0.04)
    dense = counts >= 10
    assert dense[: n - 2000].all()
    check_against_fp64(port, pos, vel, mass, prm, out, sel=dense)
    check_against_fp64(port, pos, vel, mass, prm, out, sel=~dense, acc_tau=1e-3)


@pytest.mark.parametrize("tile", [16, 24])
def test_tile_sizes(port, tile):
    w = I.scaled_dam_break(60_000, seed=24)
    out = precise_fields(w.pos, w.vel, w.mass, w.params, tile=tile)
    check_against_fp64(port, w.pos, w.vel, w.mass, w.params, out)


@pytest.mark.parametrize("max_cells", [0, 4096])
def test_folded_grid(port, max_cells):
    rng = np.random.default_rng(25)
    clusters = [np.array(c, np.float32) for c in ((0, 0, 0), (10, 10, 10), (3.3, -7.1, 0.2),
                                                   (250.0, 0.0, -40.0))]
    pos = np.concatenate([c + rng.random((3000, 3)).astype(np.float32) * 0.25
                          for c in clusters])
    n = pos.shape[0]
    vel = (0.1 * rng.standard_normal((n, 3))).astype(np.float32)
    mass = np.full(n, 1e-3, np.float32)
    prm = I.params16(xmin=-100, xmax=300, ymin=-100, ymax=100, zmin=-100, zmax=100)
    ctx = sphx.Context(n, mode=sphx.MODE_PRECISE, max_grid_cells=max_cells)
    ctx.set_params(prm)
    ctx.upload(pos, vel, mass)
    ctx.eval()
    out = ctx.download(pos=False, vel=False)
    st = ctx.stats()
    if max_cells:
        assert st["grid_cells"] <= max(max_cells, 125)
        # a 16^3 fold puts the clusters' cells in shared columns: tiles mix them and take
        # the spread launches (a CPU count of the same tiles: 64 of 712)
        assert st["spread_tiles"] > 0
    ctx.close()
    counts, _ = port.query(pos, 0.04)
    check_against_fp64(port, pos, vel, mass, prm, out, sel=counts >= 10)
    check_against_fp64(port, pos, vel, mass, prm, out, sel=counts < 10, acc_tau=1e-3)


def test_unfolded_grids_list_no_spread_tiles(built):
    """On a grid that is not folded the column runs keep every tile within 4 cells of its
    first particle's cell: no tile takes the spread launches (the dam break's sparse edge
    columns, a plain lattice, collapsed cells with a sparse rest)."""
    rng = np.random.default_rng(26)
    w = I.scaled_dam_break(60_000, seed=26)
    n = 12_000
    pos = np.empty((n, 3), np.float32)
    pos[: n - 2000] = 0.5 + 0.03 * rng.random((n - 2000, 3), dtype=np.float32)
    pos[n - 2000:] = 0.2 + 0.6 * rng.random((2000, 3), dtype=np.float32)
    lat = plain_lattice(40)
    cases = [(w.pos, w.vel, w.mass, w.params),
             (lat[0], lat[1], lat[2], I.params16()),
             (pos, np.zeros_like(pos), np.full(n, 1e-3, np.float32), I.params16())]
    for p, v, m, prm in cases:
        st = {}
        precise_fields(p, v, m, prm, stats=st)
        assert st["tiles"] > 0
        assert st["spread_tiles"] == 0, st["spread_tiles"]
