"""Generates tests/golden/sph_ref_golden.npz from the reference's own code.

Runs the reference SPH core compiled from its sources (oracle/_ref/libsph_ref.so, built by
oracle/build_ref.sh from the reference checkout) on small seeded inputs and stores inputs
and outputs as fixtures.  The fixtures travel with the repository; the reference checkout
does not.  Re-run with:  python tests/golden/make_golden.py

Cases (all arrays float32 unless noted, vectors as (n, 3)):
  lattice     8x8x8 jittered lattice (spacing 0.01, jitter 5e-4, seed 7), box [0,1]^3
  exact       6x6x6 lattice without jitter: exact ties |r| == r_search occur
  edge        hand-made: coincident pairs, NaN / inf coordinates, a far particle, particles
              outside the box, particles on cell faces, a zero-velocity-mass mix
  collapse    12x12x12 jittered lattice stepped 4 times at dt 1e-3 (the reference's
              dynamics degenerate after step 1: clamped walls, crowded cells)
  kernel/*    W / gradW / laplacianW of create_kernel(CUBIC_SPLINE | WENDLAND_C2 | GAUSSIAN,
              h = 0.02, 0.0137) at 167 vectors (zero, tiny, on q = 1 and q = 2, random)
  scene/*     the reference's initialize_dam_break / _fluid_drop / _granular_flow particle
              sets (default parameters): count, SHA-256 of (n, 11) float32 records
              pos3 vel3 mass type color3, and the first 8 records
For each case: params16, pos, vel, mass; the neighbour lists of the initial state
(counts int64, idx int32, reference order); rho/P/acc of one field evaluation (and, for
lattice / exact / edge, rho_k{1,2} / pressure_k{1,2} / acc_k{1,2}: the same evaluation
with create_kernel(WENDLAND_C2) and create_kernel(GAUSSIAN)); and for
`steps` steps of SPHEngine::step(dt) (dt > 0 fixed, dt == 0 adaptive CFL) the positions,
velocities, densities, pressures and current time after each step.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO / "sph-particle-simulator_gb300" / "python"))
sys.path.insert(0, str(REPO / "oracle"))

import sphx_inputs as I  # noqa: E402
import sph_oracle as O  # noqa: E402


def edge_case():
    pts = [
        (0.10, 0.10, 0.10), (0.10, 0.10, 0.10), (0.10, 0.10, 0.10),  # coincident triple
        (0.12, 0.10, 0.10), (0.10, 0.13, 0.10), (0.10, 0.10, 0.14),  # at <= r and = r
        (0.08, 0.08, 0.08),                                           # on a cell corner
        (0.16, 0.12, 0.04), (0.04, 0.04, 0.04),                       # cell faces (r = 0.04)
        (np.nan, 0.2, 0.2), (0.2, np.inf, 0.2), (-np.inf, 0.1, 0.1),  # non-finite
        (0.30, 0.30, 0.30), (0.32, 0.31, 0.30), (0.30, 0.33, 0.31),
        (1.5, 0.5, 0.5), (1.52, 0.5, 0.5),                            # outside the box
        (-0.2, 0.5, 0.5),
        (500.0, 500.0, 500.0), (500.01, 500.0, 500.0),                # far away
        (0.5, 0.5, 0.5), (0.5 + 0.04, 0.5, 0.5), (0.5, 0.5 + 0.039999, 0.5),
        (0.5, 0.5, 0.5 + 0.040001),
    ]
    rng = np.random.default_rng(11)
    extra = (0.6 + rng.random((24, 3)) * 0.06).tolist()
    pos = np.array(pts + extra, np.float32)
    n = pos.shape[0]
    vel = (rng.standard_normal((n, 3)) * 0.3).astype(np.float32)
    vel[3] = (np.nan, 0.0, 0.0)
    mass = np.full(n, 1e-3, np.float32)
    mass[5] = 2e-3
    prm = I.params16(xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, zmin=0.0, zmax=1.0)
    return pos, vel, mass, prm


def kernel_sample_vectors():
    """r vectors for the kernel-object fixture: zero, tiny (|r| < 1e-6), random directions
    at |r| spread over [0, 2.5h] for h = 0.02 and 0.0137, and points on q = 1 and q = 2."""
    rng = np.random.default_rng(13)
    d = rng.standard_normal((160, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rad = np.concatenate([rng.uniform(0.0, 0.05, 120), [1e-7, 5e-7, 0.0137, 0.0274, 0.02, 0.04,
                                                        0.04 + 1e-7, 0.0399999]])
    rad = np.concatenate([rad, rng.uniform(0.0, 0.05, 160 - rad.size)])
    rv = (d * rad[:, None]).astype(np.float32)
    extra = np.array([[0, 0, 0], [0.02, 0, 0], [0, 0.04, 0], [0, 0, 0.0137], [0, 0, 0.0274],
                      [1e-8, 0, 0], [0.01, 0.01, 0.01]], np.float32)
    return np.ascontiguousarray(np.concatenate([rv, extra]))


def cases():
    box = dict(xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, zmin=0.0, zmax=1.0)
    pos = I.lattice(8, 8, 8, seed=7) + np.float32(0.2)
    n = pos.shape[0]
    yield "lattice", pos, np.zeros((n, 3), np.float32), np.full(n, 1e-3, np.float32), \
        I.params16(**box), [1e-3, 1e-3, 0.0, 0.0]
    pos = I.lattice(6, 6, 6, jitter=0.0)  # on cell faces, with exact ties
    n = pos.shape[0]
    yield "exact", pos, np.zeros((n, 3), np.float32), np.full(n, 1e-3, np.float32), \
        I.params16(**box), [1e-3, 0.0]
    p, v, m, prm = edge_case()
    yield "edge", p, v, m, prm, [1e-3, 0.0, 1e-3]
    pos = I.lattice(12, 12, 12, seed=9)
    n = pos.shape[0]
    yield "collapse", pos, np.zeros((n, 3), np.float32), np.full(n, 1e-3, np.float32), \
        I.params16(**box), [1e-3, 1e-3, 1e-3, 1e-3]


def main():
    ref = O.Ref()
    out = {}
    for name, pos, vel, mass, prm, dts in cases():
        n = pos.shape[0]
        counts, idx = ref.query(pos, float(prm[15]))
        rho, P, acc = ref.fields(pos, vel, mass, prm)
        e = O.Engine(ref, n)
        e.initialize(prm)
        e.add(pos, vel, mass)
        traj = []
        for dt in dts:
            e.step(dt)
            g = e.get()
            traj.append((g["pos"], g["vel"], g["rho"], g["pressure"], e.time()))
        pre = f"{name}/"
        out[pre + "params"] = prm
        out[pre + "pos"] = pos
        out[pre + "vel"] = vel
        out[pre + "mass"] = mass
        out[pre + "counts"] = counts
        out[pre + "idx"] = idx.astype(np.int32)
        out[pre + "rho"] = rho
        out[pre + "pressure"] = P
        out[pre + "acc"] = acc
        if name != "collapse":  # the other smoothing kernels of create_kernel
            for kind in (1, 2):
                rk, Pk, ak = ref.fields(pos, vel, mass, prm, kernel=kind)
                out[pre + f"rho_k{kind}"] = rk
                out[pre + f"pressure_k{kind}"] = Pk
                out[pre + f"acc_k{kind}"] = ak
        out[pre + "dts"] = np.array(dts, np.float32)
        out[pre + "traj_pos"] = np.stack([t[0] for t in traj])
        out[pre + "traj_vel"] = np.stack([t[1] for t in traj])
        out[pre + "traj_rho"] = np.stack([t[2] for t in traj])
        out[pre + "traj_pressure"] = np.stack([t[3] for t in traj])
        out[pre + "traj_time"] = np.array([t[4] for t in traj], np.float32)
        print(f"{name}: n={n} pairs={idx.size} max|N|={counts.max()} steps={len(dts)}")
    # the reference's own scene generators, through SPHEngine::initialize_* with default
    # parameters: (n, 11) records pos3 vel3 mass type color3, pinned by SHA-256
    import ctypes as C
    import hashlib
    L = ref.lib
    L.ref_engine_particles.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_engine_init_scene.argtypes = [C.c_void_p, C.c_int]
    for which, name in enumerate(("dam_break", "fluid_drop", "granular_flow")):
        e = O.Engine(ref, 2_000_000)
        L.ref_engine_init_scene(e.h, which)
        n = e.size()
        rec = np.zeros((n, 19), np.float32)
        L.ref_engine_particles(e.h, rec.ctypes.data_as(C.c_void_p))
        rec11 = np.ascontiguousarray(np.concatenate([rec[:, 0:6], rec[:, 11:13], rec[:, 16:19]], axis=1))
        out[f"scene/{name}/n"] = np.array(n, np.int64)
        out[f"scene/{name}/sha256"] = np.frombuffer(hashlib.sha256(rec11.tobytes()).digest(), np.uint8)
        out[f"scene/{name}/first"] = rec11[:8]
        print(f"scene {name}: n={n}")
    # the kernel objects themselves: W / gradW / laplacianW of create_kernel(kind, h)
    L.ref_kernel_eval.argtypes = [C.c_int, C.c_float, C.c_size_t] + [C.c_void_p] * 4
    rv = kernel_sample_vectors()
    for kind in (0, 1, 2):
        for h in (0.02, 0.0137):
            m = rv.shape[0]
            w = np.zeros(m, np.float32)
            g = np.zeros((m, 3), np.float32)
            lap = np.zeros(m, np.float32)
            L.ref_kernel_eval(kind, C.c_float(h), m, rv.ctypes.data_as(C.c_void_p),
                              w.ctypes.data_as(C.c_void_p), g.ctypes.data_as(C.c_void_p),
                              lap.ctypes.data_as(C.c_void_p))
            key = f"kernel/k{kind}_h{h}"
            out[key + "/r"] = rv
            out[key + "/W"] = w
            out[key + "/gradW"] = g
            out[key + "/laplacianW"] = lap
    path = Path(__file__).with_name("sph_ref_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
