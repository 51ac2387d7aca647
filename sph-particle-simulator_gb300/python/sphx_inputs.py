"""Deterministic synthetic inputs for the SPH step workloads.

Every random number comes from one counter-based generator: the splitmix64 finaliser of
(seed, particle index, stream) mapped to a float32 uniform in [0, 1) with 24 random bits.
It is pure integer arithmetic, so the same seed gives the same bits on any machine, and
inputs are generated once on the host and fed to both the CPU oracle and the GPU.

Lattices follow the reference's own block generator order (src/particle.cpp:175-183):
i (x) outermost, then j (y), then k (z) innermost, i.e. index = (i*ny + j)*nz + k.

Parameter blocks are 16 float32 values in SPHParameters field order
(src/sph_engine.h:14-34):
  rest_density, gas_constant, viscosity, smoothing_length, particle_mass, timestep,
  gravity, damping, CFL_factor, xmin, xmax, ymin, ymax, zmin, zmax, neighbor_search_radius
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

PARAM_FIELDS = (
    "rest_density", "gas_constant", "viscosity", "smoothing_length", "particle_mass",
    "timestep", "gravity", "damping", "CFL_factor", "xmin", "xmax", "ymin", "ymax",
    "zmin", "zmax", "neighbor_search_radius",
)

# SPHParameters defaults (src/sph_engine.h:14-34)
DEFAULT_PARAMS = dict(
    rest_density=1000.0, gas_constant=2000.0, viscosity=0.001, smoothing_length=0.02,
    particle_mass=0.001, timestep=0.001, gravity=-9.81, damping=0.99, CFL_factor=0.4,
    xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0,
    neighbor_search_radius=0.04,
)


def params16(**overrides) -> np.ndarray:
    d = dict(DEFAULT_PARAMS)
    for k, v in overrides.items():
        if k not in d:
            raise KeyError(k)
        d[k] = v
    return np.array([d[k] for k in PARAM_FIELDS], dtype=np.float32)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = z ^ (z >> np.uint64(30))
        z = z * _M1
        z = z ^ (z >> np.uint64(27))
        z = z * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, index: np.ndarray, stream: int) -> np.ndarray:
    """float32 uniform in [0, 1) for each (seed, index, stream); stream < 8."""
    idx = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        ctr = (np.uint64(seed) << np.uint64(40)) + idx * np.uint64(8) + np.uint64(stream)
        h = _mix(ctr * _GOLDEN + _GOLDEN)
    return ((h >> np.uint64(40)).astype(np.float64) * (1.0 / 16777216.0)).astype(np.float32)


def lattice(nx: int, ny: int, nz: int, spacing: float = 0.01, jitter: float = 5e-4,
            seed: int = 0, origin=(0.0, 0.0, 0.0)) -> np.ndarray:
    """(N, 3) float32 lattice + uniform jitter in [-jitter, +jitter) per axis.

    x = origin + float32(i) * spacing + (2u - 1) * jitter, every operation in float32."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    grid = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float32)
    n = grid.shape[0]
    sp = np.float32(spacing)
    pos = grid * sp
    if jitter:
        ids = np.arange(n, dtype=np.uint64)
        jit = np.float32(jitter)
        for a in range(3):
            u = uniform(seed, ids, a)
            pos[:, a] = pos[:, a] + (u * np.float32(2.0) - np.float32(1.0)) * jit
    org = np.asarray(origin, dtype=np.float32)
    if np.any(org != 0):
        pos = pos + org
    return np.ascontiguousarray(pos, dtype=np.float32)


@dataclass
class Workload:
    """One synthetic SPH state plus the parameters and stepping it is run with."""
    name: str
    pos: np.ndarray            # (N, 3) float32
    vel: np.ndarray            # (N, 3) float32
    mass: np.ndarray           # (N,) float32
    params: np.ndarray         # (16,) float32
    dt: float                  # step size passed to step(dt); 0 = adaptive CFL
    steps: int                 # the configuration's step count
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def dam_break(nx: int, ny: int, nz: int, box, dt: float, steps: int, seed: int,
              name: str, spacing: float = 0.01, mass: float = 1e-3,
              timestep: float | None = None) -> Workload:
    pos = lattice(nx, ny, nz, spacing=spacing, jitter=5e-4, seed=seed)
    n = pos.shape[0]
    prm = params16(
        smoothing_length=0.02, neighbor_search_radius=0.04, particle_mass=mass,
        timestep=dt if timestep is None else timestep,
        xmin=box[0][0], xmax=box[0][1], ymin=box[1][0], ymax=box[1][1],
        zmin=box[2][0], zmax=box[2][1],
    )
    return Workload(name=name, pos=pos, vel=np.zeros((n, 3), np.float32),
                    mass=np.full(n, mass, np.float32), params=prm, dt=dt, steps=steps,
                    info=dict(lattice=(nx, ny, nz), spacing=spacing, seed=seed, box=box))


def config0() -> Workload:
    """Plain dam break, 10,000 particles (25x20x20), box [0,1]^3, 100 steps, dt 1e-3."""
    return dam_break(25, 20, 20, ((0, 1), (0, 1), (0, 1)), dt=1e-3, steps=100, seed=0,
                     name="dam_break_10k")


def config1() -> Workload:
    """Plain dam break, 1,000,000 particles (100^3), box [0,2]x[0,1.2]x[0,1], 100 steps,
    dt 5e-4."""
    return dam_break(100, 100, 100, ((0, 2), (0, 1.2), (0, 1)), dt=5e-4, steps=100,
                     seed=1, name="dam_break_1M")


def config4() -> Workload:
    """Large dam break, 10,000,000 particles (250x200x200), box [0,4]x[0,2.5]x[0,2],
    50 adaptive (CFL) steps capped at params.timestep = 2e-4."""
    return dam_break(250, 200, 200, ((0, 4), (0, 2.5), (0, 2)), dt=0.0, steps=50,
                     seed=4, name="dam_break_10M", timestep=2e-4)


def scaled_dam_break(n_target: int, seed: int = 1) -> Workload:
    """A config-1-like lattice block with about n_target particles (for parity tests and
    bounded CPU samples): same spacing, jitter, mass, h and box as config 1."""
    side = max(1, int(round(n_target ** (1.0 / 3.0))))
    return dam_break(side, side, side, ((0, 2), (0, 1.2), (0, 1)), dt=5e-4, steps=1,
                     seed=seed, name=f"dam_break_{side ** 3}")


def precision_cube(n: int = 1_000_000, seed: int = 2) -> Workload:
    """Config 2: n particles uniform in the cube [1000, 1001]^3, velocities N(0, 0.1^2) per
    axis (Box-Muller on the same generator), h = 0.02.  Mass gives mean density 1000 with
    the reference's kernel normalisation (its integral is 2/3): m = 1000 / (n * 2/3)."""
    ids = np.arange(n, dtype=np.uint64)
    pos = np.empty((n, 3), np.float32)
    for a in range(3):
        pos[:, a] = np.float32(1000.0) + uniform(seed, ids, a)
    vel = np.empty((n, 3), np.float32)
    for a in range(3):
        u1 = uniform(seed, ids, 3 + a).astype(np.float64)
        u2 = uniform(seed, ids, 6 if a == 0 else 7).astype(np.float64)
        if a == 2:
            u2 = 1.0 - u2
        r = np.sqrt(-2.0 * np.log(1.0 - u1))
        vel[:, a] = (0.1 * r * np.cos(2.0 * math.pi * u2)).astype(np.float32)
    m = np.float32(1000.0 / (n * (2.0 / 3.0)))
    prm = params16(smoothing_length=0.02, neighbor_search_radius=0.04, particle_mass=m,
                   xmin=1000.0, xmax=1001.0, ymin=1000.0, ymax=1001.0, zmin=1000.0,
                   zmax=1001.0)
    return Workload(name="precision_cube_1M", pos=pos, vel=vel, mass=np.full(n, m, np.float32),
                    params=prm, dt=5e-4, steps=1, info=dict(seed=seed, periodic=1.0))


@dataclass
class Batch:
    """Many independent scenes, concatenated in scene order."""
    pos: np.ndarray          # (N, 3) float32
    vel: np.ndarray          # (N, 3) float32
    mass: np.ndarray         # (N,) float32
    scene_start: np.ndarray  # (S + 1,) uint64
    params: list             # S parameter blocks
    dt: float
    steps: int
    info: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def scene(self, s: int):
        a, b = int(self.scene_start[s]), int(self.scene_start[s + 1])
        return self.pos[a:b], self.vel[a:b], self.mass[a:b], self.params[s]


def fluid_drop_scene(target: int, r_frac: float, h_frac: float, v_down: float, seed: int,
                     spacing: float = 0.01):
    """A pool filling the bottom 30% of a cubic box plus a falling sphere, on a `spacing`
    lattice with the dam break's jitter.  The box side L is chosen so that pool + sphere
    hold about `target` particles: a pool of the bottom 30% of a *unit* box alone would
    hold 300,000 particles at spacing 0.01, more than the largest scene, so the box (and
    with it the sphere: radius r_frac * L, centre height h_frac * L) is scaled per scene."""
    per_vol = 1.0 / spacing ** 3
    L = (target / (per_vol * (0.3 + 4.0 / 3.0 * math.pi * r_frac ** 3))) ** (1.0 / 3.0)
    nx = max(1, int(round(L / spacing)))
    ny = max(1, int(round(0.3 * L / spacing)))
    pool = lattice(nx, ny, nx, spacing=spacing, jitter=5e-4, seed=seed,
                   origin=(spacing / 2, spacing / 2, spacing / 2))
    R = r_frac * L
    c = np.array([L / 2, h_frac * L, L / 2])
    k = np.arange(-int(R / spacing) - 1, int(R / spacing) + 2)
    gx, gy, gz = np.meshgrid(k, k, k, indexing="ij")
    g = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1).astype(np.float64) * spacing
    sphere = (c + g[np.sum(g * g, axis=1) <= R * R]).astype(np.float32)
    pos = np.concatenate([pool, sphere]).astype(np.float32)
    vel = np.zeros_like(pos)
    vel[pool.shape[0]:, 1] = -np.float32(v_down)
    prm = params16(smoothing_length=0.02, neighbor_search_radius=0.04, particle_mass=1e-3,
                   timestep=5e-4, xmin=0.0, xmax=L, ymin=0.0, ymax=L, zmin=0.0, zmax=L)
    return pos, vel, prm, L


def fluid_drop_scene_shapes(target: int, r_frac: float, h_frac: float, v_down: float,
                            seed: int, spacing: float = 0.01) -> list:
    """The same scene as fluid_drop_scene, as two device-generator shapes (sphx_shape):
    the pool lattice and the FP64 lattice ball (same arithmetic, same order)."""
    import sphx

    per_vol = 1.0 / spacing ** 3
    L = (target / (per_vol * (0.3 + 4.0 / 3.0 * math.pi * r_frac ** 3))) ** (1.0 / 3.0)
    nx = max(1, int(round(L / spacing)))
    ny = max(1, int(round(0.3 * L / spacing)))
    org = np.float32(spacing / 2)
    pool = sphx.shape(sphx.SHAPE_LATTICE, center=(org, org, org), spacing=spacing,
                      counts=(nx, ny, nx), jitter=5e-4, seed=seed, mass=1e-3)
    R = r_frac * L
    ball = sphx.shape(sphx.SHAPE_BALL, mass=1e-3, velocity=(0.0, -np.float32(v_down), 0.0),
                      ball_center=(L / 2, h_frac * L, L / 2), ball_radius=R,
                      ball_spacing=spacing)
    return [pool, ball]


def batched_fluid_drops(nscenes: int = 256, seed: int = 3, n_min: int = 2000,
                        n_max: int = 200000) -> Batch:
    """The batched fluid-drop mix: scene sizes log-uniform in [n_min, n_max] (about 11M
    particles for 256 scenes), sphere radius U(0.05, 0.15), centre height U(0.6, 0.9) and
    downward speed U(0, 2) m/s per scene (fractions of the scene's box), dt 5e-4."""
    ids = np.arange(nscenes, dtype=np.uint64)
    u = [uniform(seed, ids, k).astype(np.float64) for k in range(4)]
    sizes = np.round(np.exp(np.log(n_min) + u[0] * (np.log(n_max) - np.log(n_min)))).astype(int)
    P, V, params, info, start = [], [], [], [], [0]
    for s in range(nscenes):
        pos, vel, prm, L = fluid_drop_scene(int(sizes[s]), 0.05 + 0.10 * u[1][s],
                                            0.6 + 0.3 * u[2][s], 2.0 * u[3][s], seed * 1000 + s)
        P.append(pos)
        V.append(vel)
        params.append(prm)
        info.append(dict(target=int(sizes[s]), n=int(pos.shape[0]), box=L,
                         args=(int(sizes[s]), 0.05 + 0.10 * u[1][s], 0.6 + 0.3 * u[2][s],
                               2.0 * u[3][s], seed * 1000 + s)))
        start.append(start[-1] + pos.shape[0])
    pos = np.concatenate(P)
    return Batch(pos=pos, vel=np.concatenate(V), mass=np.full(pos.shape[0], 1e-3, np.float32),
                 scene_start=np.array(start, np.uint64), params=params, dt=5e-4, steps=200,
                 info=info)


CONFIGS = {"dam_break_10k": config0, "dam_break_1M": config1, "dam_break_10M": config4}
