"""An application written against the reference's C++ API compiles and links unchanged
against the drop-in headers and library (CPU); on the GPU its dam-break run matches the
oracle engine bit for bit (hash of positions and densities)."""
import json
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG, REPO

APP = REPO / "tests" / "cpp" / "engine_app.cpp"


def build_app(tmp_path):
    sys.path.insert(0, str(PKG / "python"))
    import sphx_build

    sphx_build.build_host()
    exe = tmp_path / "engine_app"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(APP),
           f"-I{PKG / 'host' / 'include'}", f"-I{REPO / 'include'}",
           "-idirafter", str(PKG / "host" / "compat"), f"-L{PKG / 'lib'}", "-lsph_gb300", "-lsphx",
           f"-Wl,-rpath,{PKG / 'lib'}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_app_compiles_and_links_against_the_dropin(built, tmp_path):
    exe = build_app(tmp_path)
    assert exe.exists()


def fnv1a(h, data: bytes):
    for b in data:
        h ^= b
        h = (h * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.mark.gpu
@pytest.mark.parametrize("steps,dt", [(3, 1e-3), (2, 0.0)])
def test_app_run_matches_oracle_engine(built, port, tmp_path, steps, dt):
    import sph_oracle as O

    exe = build_app(tmp_path)
    out = subprocess.run([str(exe), str(steps), str(dt)], check=True, capture_output=True,
                         text=True).stdout
    res = json.loads(out.strip().splitlines()[-1])
    # the same scene through the oracle: the reference's generator (pybind, pinned to the
    # reference's records) and the oracle engine with the app's parameters
    sys.path.insert(0, str(PKG / "lib"))
    import sph

    p = sph.SPHParameters()
    p.bounds = [-0.25, 0.25, 0.0, 0.7, -0.45, 0.45]
    ps = sph.create_dam_break_setup([0.4, 0.6, 0.8], [0.2, 0.4, 0.8], 0.01, p)
    rec = np.ascontiguousarray(sph.particle_records(ps), np.float32)
    prm = np.array([p.rest_density, p.gas_constant, p.viscosity, p.smoothing_length,
                    p.particle_mass, p.timestep, p.gravity, p.damping, p.CFL_factor,
                    -0.25, 0.25, 0.0, 0.7, -0.45, 0.45, p.neighbor_search_radius], np.float32)
    e = O.Engine(port, 200000)
    e.initialize(prm)
    e.add(rec[:, 0:3], rec[:, 3:6], rec[:, 6])
    for _ in range(steps):
        e.step(dt)
    st = e.get()
    h = fnv1a(0xCBF29CE484222325, np.ascontiguousarray(st["pos"], np.float32).tobytes())
    h = fnv1a(h, np.ascontiguousarray(st["rho"], np.float32).tobytes())
    assert res["particles"] == rec.shape[0] and res["steps"] == steps
    assert res["hash"] == f"{h:016x}"
    assert np.float32(res["time"]) == np.float32(e.time())


@pytest.mark.parametrize("kernel", [0, 1, 2])
def test_equations_free_functions_match_the_oracle(built, port, tmp_path, kernel):
    """equations:: through the drop-in headers (host evaluation) on the reference's own
    neighbour lists: density, pressure and acceleration bit-identical to the oracle's
    evaluation of the same state (both call the C library's expf for the Gaussian)."""
    import sph_oracle as O
    import sphx_inputs as I

    sys.path.insert(0, str(PKG / "python"))
    import sphx_build

    sphx_build.build_host()
    exe = tmp_path / "equations_app"
    src = REPO / "tests" / "cpp" / "equations_app.cpp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(src),
                    f"-I{PKG / 'host' / 'include'}", f"-I{REPO / 'include'}",
                    "-idirafter", str(PKG / "host" / "compat"), f"-L{PKG / 'lib'}",
                    "-lsph_gb300", "-lsphx", f"-Wl,-rpath,{PKG / 'lib'}", "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    w = I.scaled_dam_break(3000, seed=13)
    rng = np.random.default_rng(13)
    vel = (rng.standard_normal(w.pos.shape) * 0.1).astype(np.float32)
    counts, idx = port.query(w.pos, float(w.params[15]))
    inp, outp = tmp_path / "state.bin", tmp_path / "fields.bin"
    with open(inp, "wb") as f:
        f.write(np.array([w.n], np.int64).tobytes())
        f.write(np.array([kernel], np.int32).tobytes())
        for a in (w.params, w.pos, vel, w.mass):
            f.write(np.ascontiguousarray(a, np.float32).tobytes())
        f.write(counts.astype(np.int64).tobytes())
        f.write(idx.astype(np.int64).tobytes())
    subprocess.run([str(exe), str(inp), str(outp)], check=True)
    got = np.fromfile(outp, np.float32)
    rho, P, acc = port.fields(w.pos, vel, w.mass, w.params, kernel=kernel)
    n = w.n
    for a, b, k in ((got[:n], rho, "rho"), (got[n:2 * n], P, "P"),
                    (got[2 * n:].reshape(n, 3), acc, "acc")):
        assert O.bits_equal(a, b), O.mismatch_report(a, b, k)
