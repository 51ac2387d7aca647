"""Initial conditions generated on the device.

The reference's three scenes come out of sphx_generate_scene with exactly the reference's
particle records (SHA-256 over pos, vel, mass, type, colour from the reference's own
generators, tests/golden/), and the benchmark shapes equal the host generators of
sphx_inputs.py bit for bit; a step after generation equals a step after uploading the
same particles.
"""
import hashlib

import numpy as np
import pytest

import sph_oracle as O
import sphx
import sphx_inputs as I

pytestmark = pytest.mark.gpu

# (count of the first shape, type, colour) per scene part, from the reference's generators
SCENE_PARTS = {
    "dam_break": (sphx.SCENE_DAM_BREAK, [(1, (0.5, 0.5, 0.5)), (0, (0.0, 0.5, 1.0))]),
    "fluid_drop": (sphx.SCENE_FLUID_DROP, [(0, (0.0, 0.7, 1.0))]),
    "granular_flow": (sphx.SCENE_GRANULAR_FLOW, [(1, (0.4, 0.4, 0.4)), (2, (0.8, 0.6, 0.2))]),
}


def box_count(size, sp):
    n = [int(np.float32(s) / np.float32(sp)) for s in size]
    return 2 * (n[0] * n[1] + n[1] * n[2] + n[0] * n[2])


@pytest.mark.parametrize("scene", ["dam_break", "fluid_drop", "granular_flow"])
def test_reference_scenes_match_reference_records(built, golden, scene):
    which, parts = SCENE_PARTS[scene]
    ctx = sphx.Context(200_000)
    ctx.set_params(I.params16())
    n = ctx.generate_scene(which, 0.001)
    out = ctx.download(rho=False, pressure=False, acc=False)
    assert n == int(golden[f"scene/{scene}/n"])
    rec = np.zeros((n, 11), np.float32)
    rec[:, 0:3] = out["pos"]
    rec[:, 3:6] = out["vel"]
    rec[:, 6] = 0.001
    nb = {"dam_break": box_count((0.4, 0.6, 0.8), 0.01),
          "granular_flow": box_count((1.0, 1.0, 1.0), 0.012), "fluid_drop": 0}[scene]
    bounds = [(0, nb), (nb, n)] if len(parts) == 2 else [(0, n)]
    for (a, e), (typ, col) in zip(bounds, parts):
        rec[a:e, 7] = typ
        rec[a:e, 8:11] = col
    assert np.array_equal(rec[:8].view(np.uint32), golden[f"scene/{scene}/first"].view(np.uint32))
    digest = np.frombuffer(hashlib.sha256(rec.tobytes()).digest(), np.uint8)
    assert np.array_equal(digest, golden[f"scene/{scene}/sha256"])
    ctx.close()


@pytest.mark.parametrize("dims,seed,origin", [((40, 30, 20), 1, (0.0, 0.0, 0.0)),
                                              ((17, 5, 17), 9, (0.005, 0.005, 0.005))])
def test_benchmark_lattice_matches_host_generator(built, dims, seed, origin):
    want = I.lattice(*dims, spacing=0.01, jitter=5e-4, seed=seed, origin=origin)
    ctx = sphx.Context(want.shape[0])
    ctx.set_params(I.params16())
    sh = sphx.shape(sphx.SHAPE_LATTICE, center=np.float32(origin), spacing=0.01,
                    counts=dims, jitter=5e-4, seed=seed)
    assert ctx.generate([sh]) == want.shape[0]
    got = ctx.download(vel=False, rho=False, pressure=False, acc=False)["pos"]
    assert O.bits_equal(got, want), O.mismatch_report(got, want, "pos")
    ctx.close()


def test_batched_scenes_generated_on_device_match_host(built):
    b = I.batched_fluid_drops(nscenes=4, seed=11, n_min=3000, n_max=30000)
    shapes = []
    ctx = sphx.Context(b.n)
    ctx.set_params(b.params[0])
    for s in range(4):
        shapes += I.fluid_drop_scene_shapes(*b.info[s]["args"])
    assert ctx.generate(shapes) == b.n
    out = ctx.download(rho=False, pressure=False, acc=False)
    assert O.bits_equal(out["pos"], b.pos) and O.bits_equal(out["vel"], b.vel)
    ctx.close()


def test_step_after_generate_equals_step_after_upload(built):
    w = I.scaled_dam_break(27_000, seed=3)
    outs = []
    for via in ("upload", "generate"):
        ctx = sphx.Context(w.n)
        ctx.set_params(w.params)
        if via == "upload":
            ctx.upload(w.pos, w.vel, w.mass)
        else:
            ctx.generate([sphx.shape(sphx.SHAPE_LATTICE, spacing=0.01, counts=(30, 30, 30),
                                     jitter=5e-4, seed=3, mass=1e-3)])
        ctx.step(w.dt)
        outs.append(ctx.download())
        ctx.close()
    for k in ("pos", "vel", "rho"):
        assert O.bits_equal(outs[0][k], outs[1][k]), k


def test_generate_capacity_and_precision_mode(built):
    ctx = sphx.Context(1000)
    ctx.set_params(I.params16())
    sh = sphx.shape(sphx.SHAPE_LATTICE, spacing=0.01, counts=(11, 10, 10))
    with pytest.raises(sphx.SphxError):
        ctx.generate([sh])
    assert ctx.size() == 0
    ctx.close()
    # precision mode: the lattice lands in cells + offsets; FP64 read-back = float positions
    ctx = sphx.Context(8000, mode=sphx.MODE_PRECISE)
    ctx.set_params(I.params16(xmin=0, xmax=2000, ymin=0, ymax=2000, zmin=0, zmax=2000))
    sh = sphx.shape(sphx.SHAPE_LATTICE, center=(1000.0, 1000.0, 1000.0), spacing=0.01,
                    counts=(20, 20, 20), jitter=5e-4, seed=2)
    assert ctx.generate([sh]) == 8000
    want = I.lattice(20, 20, 20, spacing=0.01, jitter=5e-4, seed=2, origin=(1000.0, 1000.0, 1000.0))
    assert np.array_equal(ctx.positions_f64(), want.astype(np.float64))
    ctx.close()
