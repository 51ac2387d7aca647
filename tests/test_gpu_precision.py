"""Precision mode (integer cell + FP32/FP16 in-cell offset, compensated sums, FP64 CFL and
time) against the FP64 oracle.

The precision study: particles uniform in a periodic cube translated to (1000, 1000,
1000) (periodicity through explicit ghost copies of the particles within r of a face),
one density + force evaluation in plain FP32 (the reference's arithmetic on float
positions), cell-offset FP32 with compensated sums, and cell-offset FP16 offsets, each
compared with an FP64 evaluation on the FP64 positions.  Stated accuracy of the FP32
cell-offset mode: density relative error <= 1e-5; acceleration error per component <=
1e-4 of the sum of the magnitudes of its terms (|a - a64| <= tau * sum_j |term_j| / m, the
cancellation-aware bound: the terms of a particle nearly cancel, so neither |a| nor the
largest |a| is a scale for its rounding error).
"""
import math

import numpy as np
import pytest

import sph_oracle as O
import sphx
import sphx_inputs as I

pytestmark = pytest.mark.gpu


def periodic_cube(n: int, side: float, origin: float, seed: int):
    """FP64 positions uniform in [origin, origin + side)^3, with ghost copies of the
    particles within r of each face (shifted by +-side), velocities N(0, 0.1^2), mass
    giving mean density 1000 with the reference kernel normalisation (integral 2/3)."""
    ids = np.arange(n, dtype=np.uint64)
    u = np.stack([I.uniform(seed, ids, a).astype(np.float64) for a in range(3)], axis=1)
    # 53-bit FP64 uniforms: combine two 24-bit draws
    u2 = np.stack([I.uniform(seed + 100, ids, a).astype(np.float64) for a in range(3)], axis=1)
    frac = (u + u2 / 16777216.0) % 1.0
    pos = origin + side * frac
    vel = np.empty((n, 3), np.float32)
    for a in range(3):
        u1 = I.uniform(seed, ids, 3 + a).astype(np.float64)
        w = I.uniform(seed, ids, 6 if a < 2 else 7).astype(np.float64)
        vel[:, a] = (0.1 * np.sqrt(-2.0 * np.log(1.0 - u1)) * np.cos(2 * math.pi * w)).astype(np.float32)
    m = np.float32(1000.0 * side ** 3 / (n * (2.0 / 3.0)))
    r = 0.04
    shifts = []
    for sx in (-1, 0, 1):
        for sy in (-1, 0, 1):
            for sz in (-1, 0, 1):
                if sx == sy == sz == 0:
                    continue
                shifts.append((sx, sy, sz))
    ghosts, gvel = [pos], [vel]
    rel = pos - origin
    for s in shifts:
        sel = np.ones(n, bool)
        for a, sa in enumerate(s):
            if sa == 1:
                sel &= rel[:, a] < r
            elif sa == -1:
                sel &= rel[:, a] >= side - r
        ghosts.append(pos[sel] + side * np.array(s, np.float64))
        gvel.append(vel[sel])
    P = np.concatenate(ghosts)
    V = np.concatenate(gvel)
    M = np.full(P.shape[0], m, np.float32)
    lo, hi = origin - 1.0, origin + side + 1.0
    prm = I.params16(smoothing_length=0.02, neighbor_search_radius=0.04, particle_mass=float(m),
                     xmin=lo, xmax=hi, ymin=lo, ymax=hi, zmin=lo, zmax=hi)
    return P, V, M, prm, n


def evaluate(mode, P64, V, M, prm):
    ctx = sphx.Context(P64.shape[0], mode=mode)
    ctx.set_params(prm)
    if mode == sphx.MODE_EXACT:
        ctx.upload(P64.astype(np.float32), V, M)
    else:
        ctx.upload_f64(P64, V, M)
    ctx.eval()
    out = ctx.download(pos=False, vel=False)
    ctx.close()
    return out


@pytest.fixture(scope="module")
def study(port):
    P, V, M, prm, n = periodic_cube(100_000, 0.464, 1000.0, seed=2)
    rho64, _, acc64, _, scale = port.fields_f64d(P, V, M, prm, want_scale=True)
    res = {}
    for name, mode in (("plain_fp32", sphx.MODE_EXACT), ("cell_fp32", sphx.MODE_PRECISE),
                       ("cell_fp16", sphx.MODE_PRECISE_FP16)):
        out = evaluate(mode, P, V, M, prm)
        rel_rho = np.abs(out["rho"][:n].astype(np.float64) - rho64[:n]) / rho64[:n]
        err = np.abs(out["acc"][:n].astype(np.float64) - acc64[:n]) / scale[:n]
        res[name] = dict(rho_max=rel_rho.max(), rho_mean=rel_rho.mean(),
                         acc_max=err.max(), acc_mean=err.mean())
    return res


def test_precision_study_errors(study):
    for k, v in study.items():
        print(k, {a: f"{b:.3e}" for a, b in v.items()})
    cell, plain, half = study["cell_fp32"], study["plain_fp32"], study["cell_fp16"]
    assert cell["rho_max"] <= 1e-5, cell
    assert cell["acc_max"] <= 1e-4, cell
    # float positions near 1000 carry ~6e-5 absolute error: plain FP32 is far worse
    assert plain["rho_max"] > 20 * cell["rho_max"]
    # binary16 offsets (~2e-5 m resolution) sit between the two
    assert half["rho_max"] > cell["rho_max"]


def test_precision_study_1M(port):
    """The configuration at full size: 1,000,000 particles in the periodic unit cube at
    (1000, 1000, 1000), one evaluation per mode; the error table goes to stdout."""
    P, V, M, prm, n = periodic_cube(1_000_000, 1.0, 1000.0, seed=2)
    rho64, _, acc64, _, scale = port.fields_f64d(P, V, M, prm, want_scale=True)
    rows = {}
    for name, mode in (("plain_fp32", sphx.MODE_EXACT), ("cell_fp32", sphx.MODE_PRECISE),
                       ("cell_fp16", sphx.MODE_PRECISE_FP16)):
        out = evaluate(mode, P, V, M, prm)
        rel = np.abs(out["rho"][:n].astype(np.float64) - rho64[:n]) / rho64[:n]
        da = np.abs(out["acc"][:n].astype(np.float64) - acc64[:n]) / scale[:n]
        rows[name] = (rel.max(), rel.mean(), da.max(), da.mean())
    print("\nprecision study 1M (errors vs FP64): rho max, rho mean, a max, a mean "
          "(acceleration errors per component over the sum of its terms' magnitudes)")
    for k, v in rows.items():
        print(f"  {k:10s} " + " ".join(f"{x:.3e}" for x in v))
    assert rows["cell_fp32"][0] <= 1e-5 and rows["cell_fp32"][2] <= 1e-4
    assert rows["plain_fp32"][0] > 20 * rows["cell_fp32"][0]


def test_precise_mode_near_origin_matches_fp64(port):
    w = I.scaled_dam_break(60_000, seed=12)
    ctx = sphx.Context(w.n, mode=sphx.MODE_PRECISE)
    ctx.set_params(w.params)
    ctx.upload(w.pos, w.vel, w.mass)
    ctx.eval()
    out = ctx.download()
    rho64, _, acc64, scale = port.fields_f64(w.pos, w.vel, w.mass, w.params, want_scale=True)
    rel = np.abs(out["rho"] - rho64) / rho64
    assert rel.max() <= 1e-5, rel.max()
    err = np.abs(out["acc"] - acc64) / np.maximum(scale, 1e-30)
    assert err.max() <= 1e-4, err.max()
    # neighbour sets: same as the reference's wherever no pair sits within 1e-6 of r
    c1, i1 = ctx.pairs()
    c2, i2 = port.query(w.pos, 0.04)
    assert np.mean(c1 == c2) > 0.999


def test_f64_round_trip_keeps_bits_far_from_origin():
    rng = np.random.default_rng(5)
    P = 1000.0 + rng.random((5000, 3))
    ctx = sphx.Context(5000, mode=sphx.MODE_PRECISE)
    ctx.set_params(I.params16(xmin=0, xmax=2000, ymin=0, ymax=2000, zmin=0, zmax=2000))
    ctx.upload_f64(P, None, np.full(5000, 1e-3, np.float32))
    back = ctx.positions_f64()
    assert np.abs(back - P).max() < 5e-9  # offset resolution, not float's 6e-5 at 1000
    # radius change re-bins the cells without losing the positions
    ctx.set_params(I.params16(neighbor_search_radius=0.05, xmin=0, xmax=2000, ymin=0,
                              ymax=2000, zmin=0, zmax=2000))
    assert np.abs(ctx.positions_f64() - P).max() < 5e-9


def test_precise_integrator_free_fall_and_walls():
    # isolated particles (no neighbours): leapfrog under gravity, cell crossings, walls
    P = np.array([[0.5, 0.5, 0.5], [3.0, 3.0, 3.0], [6.0, 0.05, 6.0]], np.float64)
    V = np.array([[0.0, 0.0, 0.0], [1.0, -2.0, 0.5], [0.0, -3.0, 0.0]], np.float32)
    M = np.full(3, 1e-3, np.float32)
    prm = I.params16(xmin=0, xmax=10, ymin=0, ymax=10, zmin=0, zmax=10, damping=1.0)
    ctx = sphx.Context(3, mode=sphx.MODE_PRECISE)
    ctx.set_params(prm)
    ctx.upload_f64(P, V, M)
    x = P.copy()
    v = V.astype(np.float64)
    dt = 0.01
    h = float(np.float32(dt))
    for _ in range(40):
        ctx.step(dt)
        a = np.array([0.0, float(np.float32(-9.81)), 0.0])
        v = v + 0.5 * a * h
        x = x + v * h
        v = v + 0.5 * a * h
        for i in range(3):  # wall at y = 0, restitution 0.8
            if x[i, 1] < 0:
                x[i, 1] = 0.0
                v[i, 1] *= -0.8
    got = ctx.positions_f64()
    assert np.abs(got - x).max() < 2e-5
    t, last = ctx.time_f64()
    dt32 = float(np.float32(dt))  # step(dt) takes a float; time accumulates it in FP64
    assert abs(t - 40 * dt32) < 1e-12 and last == dt32


def test_precise_cfl_timestep_in_fp64():
    P = np.array([[0.1, 0.1, 0.1], [0.5, 0.5, 0.5]], np.float64)
    V = np.array([[3.0, 4.0, 0.0], [0.0, 0.0, 1.0]], np.float32)
    prm = I.params16(timestep=1.0, CFL_factor=0.4, smoothing_length=0.02)
    ctx = sphx.Context(2, mode=sphx.MODE_PRECISE)
    ctx.set_params(prm)
    ctx.upload_f64(P, V, np.full(2, 1e-3, np.float32))
    ctx.step(0.0)  # first step: a0 = 0 -> dt_force = 0.4 sqrt(0.02 / 1e-6)
    _, dt = ctx.time_f64()
    cfl, h = np.float32(0.4), np.float32(0.02)
    want = min(float(cfl) * float(h) / (5.0 + 1e-6), float(cfl) * math.sqrt(float(h) / 1e-6), 1.0)
    assert dt == pytest.approx(want, rel=1e-12)
