"""Headless rendering: the reference's billboard shader pair as CUDA kernels.

The instance buffer (clip-space quad corners + fragment colour) and the rasterised RGBA
image must equal, bit for bit, the CPU restatement in oracle/render_oracle.c, which fixes
the shader arithmetic's evaluation order and the rasterisation rules (pixel centres,
top-left ties, GL_LESS in draw order).  The reference's own GL output cannot be produced
on these machines, so the restatement is pinned to the shader source only.
"""
import numpy as np
import pytest

import sphx
import sphx_inputs as I

pytestmark = pytest.mark.gpu


def setup_ctx(w, mode=sphx.MODE_EXACT):
    ctx = sphx.Context(w.n, mode=mode)
    ctx.set_params(w.params)
    ctx.upload(w.pos, w.vel, w.mass)
    return ctx


def cameras():
    yield sphx.camera_matrices()                                    # the Camera defaults
    yield sphx.camera_matrices((0.5, 0.4, 2.0), -90.0, 0.0, 45.0, 16 / 9)   # main.cpp's view
    yield sphx.camera_matrices((1.8, 1.2, 1.6), -135.0, -25.0, 35.0, 4 / 3)


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_instances_match_oracle(built, port, mode):
    w = I.config0()
    rng = np.random.default_rng(3)
    w.vel[:] = rng.standard_normal(w.vel.shape).astype(np.float32)
    colors = rng.random((w.n, 3)).astype(np.float32)
    ctx = setup_ctx(w)
    for view, proj in cameras():
        rp = sphx.render_params(view, proj, particle_size=0.01, color_mode=mode)
        got = ctx.render_instances(rp, colors if mode == 3 else None)
        want = port.render_instances(rp, w.pos, w.vel, colors if mode == 3 else None)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    ctx.close()


@pytest.mark.parametrize("size", [(320, 180), (1280, 720)])
def test_image_matches_oracle(built, port, size):
    w = I.scaled_dam_break(60_000, seed=4)
    rng = np.random.default_rng(5)
    w.vel[:] = (rng.standard_normal(w.vel.shape) * 0.8).astype(np.float32)
    colors = rng.random((w.n, 3)).astype(np.float32)
    ctx = setup_ctx(w)
    for mode in (0, 3):
        for view, proj in cameras():
            rp = sphx.render_params(view, proj, particle_size=0.005, color_mode=mode,
                                    width=size[0], height=size[1])
            col = colors if mode == 3 else None
            got = ctx.render_image(rp, col)
            want = port.render_image(rp, w.pos, w.vel, col)
            bad = np.argwhere(np.any(got != want, axis=2))
            assert bad.size == 0, f"{len(bad)} pixels differ, first {bad[:3].tolist()}"
    # something was drawn, and the background elsewhere
    bg = np.array([26, 26, 38, 255], np.uint8)  # round((0.1, 0.1, 0.15) * 255)
    assert (got != bg).any(axis=2).mean() > 0.01 and (got == bg).all(axis=2).mean() > 0.1
    ctx.close()


def test_depth_order_and_ties(built, port):
    # two stacks of particles on the view axis: the nearest wins; identical positions
    # (equal depth) keep the first-drawn particle, as GL_LESS does
    pos = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.5], [0.0, 0.0, 0.5], [0.3, 0.0, 0.2],
                    [0.3, 0.0, 0.2], [0.3, 0.0, -0.4]], np.float32)
    vel = np.zeros_like(pos)
    colors = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [0, 1, 1], [1, 0, 1]],
                      np.float32)
    ctx = sphx.Context(len(pos))
    ctx.set_params(I.params16())
    ctx.upload(pos, vel, np.full(len(pos), 1e-3, np.float32))
    view, proj = sphx.camera_matrices((0.0, 0.0, 3.0))
    rp = sphx.render_params(view, proj, particle_size=0.1, color_mode=3, width=200, height=200)
    got = ctx.render_image(rp, colors)
    want = port.render_image(rp, pos, vel, colors)
    assert np.array_equal(got, want)
    centre = got[100, 100, :3].astype(int)
    assert centre[1] > centre[0] and centre[1] > centre[2]  # particle 1 (green) wins
    ctx.close()


def test_precision_mode_renders_cell_offset_positions(built, port):
    P = 1000.0 + np.random.default_rng(8).random((4000, 3)) * 0.5
    ctx = sphx.Context(len(P), mode=sphx.MODE_PRECISE)
    ctx.set_params(I.params16(xmin=0, xmax=2000, ymin=0, ymax=2000, zmin=0, zmax=2000))
    vel = np.zeros((len(P), 3), np.float32)
    ctx.upload_f64(P, vel, np.full(len(P), 1e-3, np.float32))
    view, proj = sphx.camera_matrices((1000.25, 1000.25, 1002.0))
    rp = sphx.render_params(view, proj, particle_size=0.004, color_mode=1, width=256, height=256)
    pos32 = ctx.positions_f64().astype(np.float32)
    assert np.array_equal(ctx.render_instances(rp).view(np.uint32),
                          port.render_instances(rp, pos32, vel).view(np.uint32))
    assert np.array_equal(ctx.render_image(rp), port.render_image(rp, pos32, vel))
    ctx.close()


def test_device_entry_points_and_empty_scene(built):
    torch = pytest.importorskip("torch")
    w = I.config0()
    ctx = setup_ctx(w)
    view, proj = sphx.camera_matrices((0.5, 0.4, 2.0))
    rp = sphx.render_params(view, proj, color_mode=0, width=64, height=48)
    host = ctx.render_instances(rp)
    dev = torch.empty((w.n, 20), dtype=torch.float32, device="cuda")
    lib = sphx.lib()
    import ctypes as C
    assert lib.sphx_render_instances_device(ctx._h, C.byref(rp), None,
                                            C.c_void_p(dev.data_ptr())) == 0
    img_dev = torch.empty((48, 64, 4), dtype=torch.uint8, device="cuda")
    assert lib.sphx_render_image_device(ctx._h, C.byref(rp), None,
                                        C.c_void_p(img_dev.data_ptr())) == 0
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), host.view(np.uint32))
    assert np.array_equal(img_dev.cpu().numpy(), ctx.render_image(rp))
    ctx.close()
    empty = sphx.Context(16)
    empty.set_params(I.params16())
    img = empty.render_image(rp)
    assert (img == np.array([26, 26, 38, 255], np.uint8)).all()
    bad = sphx.render_params(view, proj, color_mode=7)
    with pytest.raises(sphx.SphxError):
        empty.render_image(bad)
    empty.close()
