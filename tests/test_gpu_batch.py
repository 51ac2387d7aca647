"""Batched scenes: many independent scenes advanced by one launch sequence.

Every scene must come out bit-identical to the same scene stepped alone through the
plain step (which is itself bit-identical to the reference), for fixed and adaptive dt,
eagerly or through the captured CUDA graph; per-scene time, dt and FP64 sums likewise.
"""
import numpy as np
import pytest

import sph_oracle as O
import sphx
import sphx_inputs as I

pytestmark = pytest.mark.gpu


def small_batch(nscenes=10):
    return I.batched_fluid_drops(nscenes=nscenes, seed=7, n_min=500, n_max=20000)


def run_alone(b, s, dts):
    pos, vel, mass, prm = b.scene(s)
    ctx = sphx.Context(max(pos.shape[0], 1))
    ctx.set_params(prm)
    ctx.upload(pos, vel, mass)
    for dt in dts:
        ctx.step(dt)
    out = ctx.download(acc=False)
    t, last = ctx.time()
    st = ctx.stats()
    ctx.close()
    return out, t, last, st


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("dts", [[5e-4] * 3, [0.0] * 3])
def test_batch_matches_scenes_stepped_alone(graph, dts):
    b = small_batch()
    ctx = sphx.Context(b.n, graph=graph)
    ctx.upload(b.pos, b.vel, b.mass)
    ctx.set_scenes(b.scene_start, b.params)
    for dt in dts:
        ctx.step(dt)
    out = ctx.download(acc=False)
    for s in range(len(b.params)):
        a, e = int(b.scene_start[s]), int(b.scene_start[s + 1])
        ref, t, last, st = run_alone(b, s, dts)
        for k in ("pos", "vel", "rho", "pressure"):
            assert O.bits_equal(out[k][a:e], ref[k]), O.mismatch_report(out[k][a:e], ref[k], f"{k} scene {s}")
        sc = ctx.scene_stats(s)
        assert sc["current_time"] == t and sc["last_dt"] == last
        assert sc["count"] == e - a
        assert sc["sum_mass"] == pytest.approx(st["sum_mass"], rel=1e-12)
        assert sc["kinetic_energy"] == pytest.approx(st["kinetic_energy"], rel=1e-9)


def test_graph_replay_equals_eager_over_many_steps():
    b = small_batch(6)
    outs = []
    for graph in (False, True):
        ctx = sphx.Context(b.n, graph=graph)
        ctx.upload(b.pos, b.vel, b.mass)
        ctx.set_scenes(b.scene_start, b.params)
        for _ in range(8):
            ctx.step(0.0)
        outs.append(ctx.download(acc=False))
        ctx.close()
    for k in ("pos", "vel", "rho"):
        assert O.bits_equal(outs[0][k], outs[1][k]), k


def test_single_scene_graph_matches_eager(port):
    w = I.config0()
    res = []
    for graph in (False, True):
        ctx = sphx.Context(w.n, graph=graph)
        ctx.set_params(w.params)
        ctx.upload(w.pos, w.vel, w.mass)
        for dt in (1e-3, 1e-3, 0.0, 0.0, 1e-3):
            ctx.step(dt)
        res.append(ctx.download())
        ctx.close()
    for k in ("pos", "vel", "rho", "acc"):
        assert O.bits_equal(res[0][k], res[1][k]), k


def test_autotune_keeps_state_and_results():
    b = small_batch(8)
    ctx = sphx.Context(b.n)
    ctx.upload(b.pos, b.vel, b.mass)
    ctx.set_scenes(b.scene_start, b.params)
    w, bps, ms = ctx.autotune(5e-4)
    assert w in (1, 2, 4) and ms > 0
    assert ctx.tuning()["tile_particles"] in (16, 24, 32)
    assert np.array_equal(ctx.download(vel=False, rho=False, pressure=False, acc=False)["pos"], b.pos)
    ctx.step(5e-4)
    tuned = ctx.download(acc=False)
    ref = sphx.Context(b.n)
    ref.upload(b.pos, b.vel, b.mass)
    ref.set_scenes(b.scene_start, b.params)
    ref.step(5e-4)
    plain = ref.download(acc=False)
    for k in ("pos", "vel", "rho"):
        assert O.bits_equal(tuned[k], plain[k]), k
    assert ctx.scene_stats(0)["current_time"] == np.float32(5e-4)


def test_scene_validation():
    b = small_batch(3)
    ctx = sphx.Context(b.n)
    ctx.upload(b.pos, b.vel, b.mass)
    bad = b.scene_start.copy()
    bad[-1] -= 1  # does not cover the particle set
    with pytest.raises(sphx.SphxError):
        ctx.set_scenes(bad, b.params)
    pctx = sphx.Context(b.n, mode=sphx.MODE_PRECISE)
    pctx.set_params(b.params[0])
    pctx.upload(b.pos, b.vel, b.mass)
    with pytest.raises(sphx.SphxError):  # exact mode only
        pctx.set_scenes(b.scene_start, b.params)


def test_batch_scenes_match_the_oracle_directly(port):
    """Every scene of a batched step against the oracle engine stepping that scene alone
    (fixed and CFL dt): positions, velocities, densities and pressures bit-identical."""
    b = small_batch(5)
    for dts in ([5e-4, 5e-4], [0.0, 0.0]):
        ctx = sphx.Context(b.n)
        ctx.upload(b.pos, b.vel, b.mass)
        ctx.set_scenes(b.scene_start, b.params)
        for dt in dts:
            ctx.step(dt)
        out = ctx.download(acc=False)
        ctx.close()
        for s in range(len(b.params)):
            a, e = int(b.scene_start[s]), int(b.scene_start[s + 1])
            pos, vel, mass, prm = b.scene(s)
            eng = O.Engine(port, pos.shape[0])
            eng.initialize(prm)
            eng.add(pos, vel, mass)
            for dt in dts:
                eng.step(dt)
            ref = eng.get()
            for k in ("pos", "vel", "rho", "pressure"):
                assert O.bits_equal(out[k][a:e], ref[k]), O.mismatch_report(
                    out[k][a:e], ref[k], f"{k} scene {s} dts {dts}")
