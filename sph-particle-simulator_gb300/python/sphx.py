"""ctypes binding of the sphx C ABI (include/sphx.h).

This is how Python callers -- the tests, the bench and the smoke check -- drive the GPU
step through exactly the entry points a C/C++ host binds.  The shared library is the
in-tree build <package>/lib/libsphx.so; if it is missing the import fails loudly: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parents[1]
LIB_PATH = Path(os.environ.get("SPHX_LIB", _PKG / "lib" / "libsphx.so"))

OK = 0
ERRORS = {
    -1: "SPHX_ERR_INVALID_ARG", -2: "SPHX_ERR_OOM", -3: "SPHX_ERR_CUDA",
    -4: "SPHX_ERR_TIMEOUT", -5: "SPHX_ERR_CAPACITY", -6: "SPHX_ERR_NOT_READY",
    -7: "SPHX_ERR_DOMAIN", -8: "SPHX_ERR_OVERFLOW",
}
MODE_EXACT = 0
MODE_PRECISE = 1
MODE_PRECISE_FP16 = 2
# smoothing kernels (sph::KernelType order)
KERNEL_CUBIC_SPLINE = 0
KERNEL_WENDLAND_C2 = 1
KERNEL_GAUSSIAN = 2
# render colour modes (RenderParameters::ColorMode order)
COLOR_VELOCITY, COLOR_DENSITY, COLOR_PRESSURE, COLOR_TYPE = 0, 1, 2, 3
# device generation (sphx_shape kinds, reference scenes)
SHAPE_BLOCK, SHAPE_BOX, SHAPE_SPHERE, SHAPE_LATTICE, SHAPE_BALL = 0, 1, 2, 3, 4
SCENE_DAM_BREAK, SCENE_FLUID_DROP, SCENE_GRANULAR_FLOW = 0, 1, 2

# every symbol include/sphx.h declares
EXPORTS = (
    "sphx_version", "sphx_strerror", "sphx_create", "sphx_destroy", "sphx_set_stream",
    "sphx_set_params", "sphx_upload", "sphx_upload_f64", "sphx_step", "sphx_eval",
    "sphx_download", "sphx_download_f64", "sphx_get_time_f64",
    "sphx_size", "sphx_get_time", "sphx_set_time", "sphx_get_stats", "sphx_reset_stats",
    "sphx_snapshot", "sphx_restore", "sphx_debug_pairs", "sphx_debug_pairs_subset",
    "sphx_grid_create",
    "sphx_grid_destroy", "sphx_grid_build", "sphx_grid_query", "sphx_grid_info",
    "sphx_grid_cell", "sphx_set_scenes", "sphx_get_scene_stats", "sphx_autotune",
    "sphx_density_noalloc", "sphx_get_tuning", "sphx_alloc_host", "sphx_free_host",
    "sphx_set_kernel", "sphx_get_kernel", "sphx_camera_matrices",
    "sphx_render_instances", "sphx_render_instances_device", "sphx_render_image",
    "sphx_render_image_device", "sphx_generate", "sphx_generate_scene",
)
NOALLOC_MAX_PARTICLES = 65536


class SphxParams(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "rest_density", "gas_constant", "viscosity", "smoothing_length", "particle_mass",
        "timestep", "gravity", "damping", "cfl_factor", "xmin", "xmax", "ymin", "ymax",
        "zmin", "zmax", "neighbor_search_radius")]


class SphxTuning(C.Structure):
    _fields_ = [("mode", C.c_int), ("warps_per_block", C.c_int), ("blocks_per_sm", C.c_int),
                ("max_grid_cells", C.c_int64), ("profile", C.c_int), ("graph", C.c_int),
                ("tile_particles", C.c_int), ("bulk_copy", C.c_int)]


class SphxSceneStats(C.Structure):
    _fields_ = [("start", C.c_uint64), ("count", C.c_uint64), ("current_time", C.c_float),
                ("last_dt", C.c_float), ("grid_cells", C.c_uint32), ("pad", C.c_uint32),
                ("sum_mass", C.c_double), ("momentum", C.c_double * 3),
                ("kinetic_energy", C.c_double), ("potential_energy", C.c_double)]


class SphxStats(C.Structure):
    _fields_ = [
        ("total_time", C.c_double), ("neighbor_search_time", C.c_double),
        ("density_computation_time", C.c_double), ("force_computation_time", C.c_double),
        ("integration_time", C.c_double), ("max_neighbors", C.c_uint64),
        ("total_neighbor_queries", C.c_uint64), ("steps", C.c_uint64),
        ("current_time", C.c_float), ("last_dt", C.c_float),
        ("occupied_cells", C.c_uint32), ("max_cell_occupancy", C.c_uint32),
        ("nonfinite_particles", C.c_uint32), ("grid_cells", C.c_uint32),
        ("sum_mass", C.c_double), ("momentum", C.c_double * 3),
        ("kinetic_energy", C.c_double), ("potential_energy", C.c_double),
        ("sum_density", C.c_double), ("kernel_launches", C.c_uint64),
        ("tiles", C.c_uint32), ("spread_tiles", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name == "momentum" else v
        return d


class SphxShape(C.Structure):
    """sphx_shape: one primitive of a device-generated particle set."""
    _fields_ = [("kind", C.c_int), ("center", C.c_float * 3), ("size", C.c_float * 3),
                ("spacing", C.c_float), ("mass", C.c_float), ("velocity", C.c_float * 3),
                ("counts", C.c_int * 3), ("jitter", C.c_float), ("seed", C.c_uint64),
                ("ball_center", C.c_double * 3), ("ball_radius", C.c_double),
                ("ball_spacing", C.c_double)]


def shape(kind, center=(0.0, 0.0, 0.0), size=(0.0, 0.0, 0.0), spacing=0.01, mass=1e-3,
          velocity=(0.0, 0.0, 0.0), counts=(0, 0, 0), jitter=0.0, seed=0,
          ball_center=(0.0, 0.0, 0.0), ball_radius=0.0, ball_spacing=0.0) -> SphxShape:
    s = SphxShape()
    s.kind = kind
    s.center[:] = [float(x) for x in center]
    s.size[:] = [float(x) for x in size]
    s.spacing, s.mass = spacing, mass
    s.velocity[:] = [float(x) for x in velocity]
    s.counts[:] = [int(x) for x in counts]
    s.jitter, s.seed = jitter, int(seed)
    s.ball_center[:] = [float(x) for x in ball_center]
    s.ball_radius, s.ball_spacing = float(ball_radius), float(ball_spacing)
    return s


class SphxRenderParams(C.Structure):
    """sphx_render_params: column-major view / projection / model, particle size, colour
    mode, image size, background colour."""
    _fields_ = [("view", C.c_float * 16), ("projection", C.c_float * 16),
                ("model", C.c_float * 16), ("particle_size", C.c_float),
                ("color_mode", C.c_int), ("width", C.c_int), ("height", C.c_int),
                ("background", C.c_float * 3)]


def camera_matrices(position=(0.0, 0.0, 3.0), yaw=-90.0, pitch=0.0, fov=45.0,
                    aspect=1280 / 720):
    """view, projection (16 float32 each, column-major) of the reference's Camera
    (src/renderer.h:16-29, renderer.cpp:12-29) -- defaults are its defaults."""
    v = (C.c_float * 16)()
    p = (C.c_float * 16)()
    pos = (C.c_float * 3)(*position)
    lib().sphx_camera_matrices(pos, C.c_float(yaw), C.c_float(pitch), C.c_float(fov),
                               C.c_float(aspect), v, p)
    return np.frombuffer(v, np.float32).copy(), np.frombuffer(p, np.float32).copy()


def render_params(view, projection, model=None, particle_size=0.01, color_mode=0,
                  width=1280, height=720, background=(0.1, 0.1, 0.15)) -> SphxRenderParams:
    """Render parameters (defaults: the reference's RenderParameters, src/renderer.h:32-56)."""
    rp = SphxRenderParams()
    rp.view[:] = [float(x) for x in np.asarray(view, np.float32).ravel()]
    rp.projection[:] = [float(x) for x in np.asarray(projection, np.float32).ravel()]
    m = np.eye(4, dtype=np.float32) if model is None else np.asarray(model, np.float32)
    rp.model[:] = [float(x) for x in m.ravel()]
    rp.particle_size = particle_size
    rp.color_mode = color_mode
    rp.width, rp.height = width, height
    rp.background[:] = [float(x) for x in background]
    return rp


class SphxError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where}: {ERRORS.get(code, code)} ({code})")
        self.code = code


def load_library(path: Path | str = LIB_PATH) -> C.CDLL:
    path = Path(path)
    if not path.exists():
        raise ImportError(f"sphx CUDA library not built: {path} (run __graft_entry__.build())")
    lib = C.CDLL(str(path))
    vp, sz, fp = C.c_void_p, C.c_size_t, C.c_void_p
    sig = {
        "sphx_version": ([], C.c_int),
        "sphx_strerror": ([C.c_int], C.c_char_p),
        "sphx_create": ([C.POINTER(vp), sz, C.POINTER(SphxTuning)], C.c_int),
        "sphx_destroy": ([vp], None),
        "sphx_set_stream": ([vp, vp], C.c_int),
        "sphx_set_params": ([vp, C.POINTER(SphxParams)], C.c_int),
        "sphx_set_kernel": ([vp, C.c_int], C.c_int),
        "sphx_camera_matrices": ([fp, C.c_float, C.c_float, C.c_float, C.c_float, fp, fp], None),
        "sphx_generate": ([vp, sz, C.POINTER(SphxShape), C.POINTER(sz)], C.c_int),
        "sphx_generate_scene": ([vp, C.c_int, C.c_float, C.POINTER(sz)], C.c_int),
        "sphx_render_instances": ([vp, C.POINTER(SphxRenderParams), fp, fp], C.c_int),
        "sphx_render_instances_device": ([vp, C.POINTER(SphxRenderParams), fp, fp], C.c_int),
        "sphx_render_image": ([vp, C.POINTER(SphxRenderParams), fp, fp], C.c_int),
        "sphx_render_image_device": ([vp, C.POINTER(SphxRenderParams), fp, fp], C.c_int),
        "sphx_get_kernel": ([vp, C.POINTER(C.c_int)], C.c_int),
        "sphx_upload": ([vp, sz, fp, fp, fp], C.c_int),
        "sphx_upload_f64": ([vp, sz, fp, fp, fp], C.c_int),
        "sphx_download_f64": ([vp, fp], C.c_int),
        "sphx_get_time_f64": ([vp, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "sphx_step": ([vp, C.c_float], C.c_int),
        "sphx_eval": ([vp], C.c_int),
        "sphx_download": ([vp, fp, fp, fp, fp, fp], C.c_int),
        "sphx_size": ([vp, C.POINTER(sz)], C.c_int),
        "sphx_get_time": ([vp, C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
        "sphx_set_time": ([vp, C.c_float], C.c_int),
        "sphx_get_stats": ([vp, C.POINTER(SphxStats)], C.c_int),
        "sphx_reset_stats": ([vp], C.c_int),
        "sphx_snapshot": ([vp], C.c_int),
        "sphx_restore": ([vp], C.c_int),
        "sphx_debug_pairs": ([vp, fp, fp, C.POINTER(sz)], C.c_int),
        "sphx_debug_pairs_subset": ([vp, sz, fp, fp, fp, C.POINTER(sz)], C.c_int),
        "sphx_density_noalloc": ([C.POINTER(SphxParams), sz, fp, fp, fp, fp, vp], C.c_int),
        "sphx_set_scenes": ([vp, C.c_uint32, fp, C.POINTER(SphxParams)], C.c_int),
        "sphx_get_scene_stats": ([vp, C.c_uint32, C.POINTER(SphxSceneStats)], C.c_int),
        "sphx_get_tuning": ([vp, C.POINTER(SphxTuning)], C.c_int),
        "sphx_autotune": ([vp, C.c_float, C.POINTER(C.c_int), C.POINTER(C.c_int),
                           C.POINTER(C.c_float)], C.c_int),
        "sphx_grid_create": ([C.POINTER(vp), sz], C.c_int),
        "sphx_grid_destroy": ([vp], None),
        "sphx_grid_build": ([vp, sz, fp, C.c_float], C.c_int),
        "sphx_grid_query": ([vp, sz, fp, C.c_float, fp, fp, C.POINTER(sz)], C.c_int),
        "sphx_grid_info": ([vp, C.POINTER(sz), C.POINTER(sz)], C.c_int),
        "sphx_grid_cell": ([vp, C.c_int, C.c_int, C.c_int, fp, C.POINTER(sz)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


_LIB: C.CDLL | None = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load_library()
    return _LIB


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a, shape_last=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a


def params_struct(p16) -> SphxParams:
    p = np.asarray(p16, dtype=np.float32).ravel()
    if p.size != 16:
        raise ValueError("a parameter block has 16 floats")
    return SphxParams(*[float(x) for x in p])


class Context:
    """One sphx context (one GPU step engine)."""

    def __init__(self, capacity: int, *, mode: int = MODE_EXACT, warps_per_block: int = 0,
                 blocks_per_sm: int = 0, max_grid_cells: int = 0, profile: bool = False,
                 graph: bool = False, tile_particles: int = 0, bulk_copy: bool = False):
        self._lib = lib()
        self._h = C.c_void_p()
        t = SphxTuning(mode, warps_per_block, blocks_per_sm, max_grid_cells, int(profile),
                       int(graph), tile_particles, int(bulk_copy))
        self._check(self._lib.sphx_create(C.byref(self._h), capacity, C.byref(t)), "sphx_create")
        self.capacity = capacity

    def _check(self, rc: int, where: str):
        if rc != OK:
            raise SphxError(rc, where)

    def close(self):
        if self._h:
            self._lib.sphx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr: int | None):
        self._check(self._lib.sphx_set_stream(self._h, stream_ptr or None), "sphx_set_stream")

    def generate(self, shapes) -> int:
        """Replaces the particle set with the shapes' particles, generated on the GPU."""
        arr = (SphxShape * max(len(shapes), 1))(*shapes)
        n = C.c_size_t(0)
        self._check(self._lib.sphx_generate(self._h, len(shapes), arr, C.byref(n)),
                    "sphx_generate")
        return n.value

    def generate_scene(self, scene: int, particle_mass: float = 1e-3) -> int:
        """The reference's initialize_dam_break / _fluid_drop / _granular_flow particle set."""
        n = C.c_size_t(0)
        self._check(self._lib.sphx_generate_scene(self._h, int(scene), C.c_float(particle_mass),
                                                  C.byref(n)), "sphx_generate_scene")
        return n.value

    def render_instances(self, rp: SphxRenderParams, colors=None) -> np.ndarray:
        """(n, 20) float32: 4 clip-space corners (x, y, z, w) and RGBA per particle."""
        n = self.size()
        out = np.zeros((n, 20), np.float32)
        col = None if colors is None else np.ascontiguousarray(colors, np.float32).reshape(n, 3)
        self._check(self._lib.sphx_render_instances(self._h, C.byref(rp), _ptr(col), _ptr(out)),
                    "sphx_render_instances")
        return out

    def render_image(self, rp: SphxRenderParams, colors=None) -> np.ndarray:
        """(height, width, 4) uint8 RGBA image, rows bottom-up (GL order)."""
        n = self.size()
        img = np.zeros((rp.height, rp.width, 4), np.uint8)
        col = None if colors is None else np.ascontiguousarray(colors, np.float32).reshape(n, 3)
        self._check(self._lib.sphx_render_image(self._h, C.byref(rp), _ptr(col), _ptr(img)),
                    "sphx_render_image")
        return img

    def set_kernel(self, kernel: int):
        """Smoothing kernel of the passes: KERNEL_CUBIC_SPLINE (the reference engine's),
        KERNEL_WENDLAND_C2 or KERNEL_GAUSSIAN (create_kernel, src/kernels.cpp:226-236)."""
        self._check(self._lib.sphx_set_kernel(self._h, int(kernel)), "sphx_set_kernel")

    def kernel(self) -> int:
        k = C.c_int(0)
        self._check(self._lib.sphx_get_kernel(self._h, C.byref(k)), "sphx_get_kernel")
        return k.value

    def set_params(self, p16):
        self._check(self._lib.sphx_set_params(self._h, C.byref(params_struct(p16))),
                    "sphx_set_params")

    def upload(self, pos, vel=None, mass=None):
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = None if vel is None else _f32(vel).reshape(n, 3)
        mass = _f32(mass).reshape(n)
        self._keep = (pos, vel, mass)
        self._check(self._lib.sphx_upload(self._h, n, _ptr(pos), _ptr(vel), _ptr(mass)),
                    "sphx_upload")

    def upload_f64(self, pos64, vel=None, mass=None):
        pos64 = np.ascontiguousarray(pos64, np.float64).reshape(-1, 3)
        n = pos64.shape[0]
        vel = None if vel is None else _f32(vel).reshape(n, 3)
        mass = _f32(mass).reshape(n)
        self._keep = (pos64, vel, mass)
        self._check(self._lib.sphx_upload_f64(self._h, n, _ptr(pos64), _ptr(vel), _ptr(mass)),
                    "sphx_upload_f64")

    def positions_f64(self) -> np.ndarray:
        out = np.empty((self.size(), 3), np.float64)
        self._check(self._lib.sphx_download_f64(self._h, _ptr(out)), "sphx_download_f64")
        return out

    def time_f64(self) -> tuple[float, float]:
        t, dt = C.c_double(), C.c_double()
        self._check(self._lib.sphx_get_time_f64(self._h, C.byref(t), C.byref(dt)), "sphx_get_time_f64")
        return t.value, dt.value

    def set_scenes(self, scene_start, params_list):
        """Split the loaded particles into scenes (contiguous ranges) with their parameters."""
        ss = np.ascontiguousarray(scene_start, np.uint64)
        k = ss.size - 1
        arr = (SphxParams * max(k, 1))(*[params_struct(p) for p in params_list])
        self._check(self._lib.sphx_set_scenes(self._h, k, _ptr(ss), arr), "sphx_set_scenes")

    def autotune(self, dt: float) -> tuple[int, int, float]:
        w, b, ms = C.c_int(), C.c_int(), C.c_float()
        self._check(self._lib.sphx_autotune(self._h, C.c_float(dt), C.byref(w), C.byref(b),
                                            C.byref(ms)), "sphx_autotune")
        return w.value, b.value, ms.value

    def tuning(self) -> dict:
        """The context's launch shape and options (after creation or autotune)."""
        t = SphxTuning()
        self._check(self._lib.sphx_get_tuning(self._h, C.byref(t)), "sphx_get_tuning")
        return {name: getattr(t, name) for name, _ in t._fields_}

    def scene_stats(self, scene: int) -> dict:
        st = SphxSceneStats()
        self._check(self._lib.sphx_get_scene_stats(self._h, scene, C.byref(st)),
                    "sphx_get_scene_stats")
        d = {name: getattr(st, name) for name, _ in st._fields_ if name != "pad"}
        d["momentum"] = list(st.momentum)
        return d

    def upload_ptr(self, n: int, pos_ptr: int, vel_ptr: int | None, mass_ptr: int):
        """Upload from raw host pointers (e.g. pinned buffers)."""
        self._check(self._lib.sphx_upload(self._h, n, C.c_void_p(pos_ptr),
                                          C.c_void_p(vel_ptr) if vel_ptr else None,
                                          C.c_void_p(mass_ptr)), "sphx_upload")

    def step(self, dt: float = 0.0):
        self._check(self._lib.sphx_step(self._h, C.c_float(dt)), "sphx_step")

    def eval(self):
        self._check(self._lib.sphx_eval(self._h), "sphx_eval")

    def size(self) -> int:
        n = C.c_size_t()
        self._check(self._lib.sphx_size(self._h, C.byref(n)), "sphx_size")
        return n.value

    def download(self, pos=True, vel=True, rho=True, pressure=True, acc=True) -> dict:
        n = self.size()
        out = {}
        if pos:
            out["pos"] = np.empty((n, 3), np.float32)
        if vel:
            out["vel"] = np.empty((n, 3), np.float32)
        if rho:
            out["rho"] = np.empty(n, np.float32)
        if pressure:
            out["pressure"] = np.empty(n, np.float32)
        if acc:
            out["acc"] = np.empty((n, 3), np.float32)
        self._check(self._lib.sphx_download(
            self._h, _ptr(out.get("pos")), _ptr(out.get("vel")), _ptr(out.get("rho")),
            _ptr(out.get("pressure")), _ptr(out.get("acc"))), "sphx_download")
        return out

    def download_ptr(self, pos_ptr, vel_ptr, rho_ptr, p_ptr, acc_ptr):
        cv = lambda p: C.c_void_p(p) if p else None
        self._check(self._lib.sphx_download(self._h, cv(pos_ptr), cv(vel_ptr), cv(rho_ptr),
                                            cv(p_ptr), cv(acc_ptr)), "sphx_download")

    def time(self) -> tuple[float, float]:
        t, dt = C.c_float(), C.c_float()
        self._check(self._lib.sphx_get_time(self._h, C.byref(t), C.byref(dt)), "sphx_get_time")
        return t.value, dt.value

    def set_time(self, t: float):
        self._check(self._lib.sphx_set_time(self._h, C.c_float(t)), "sphx_set_time")

    def stats(self) -> dict:
        s = SphxStats()
        self._check(self._lib.sphx_get_stats(self._h, C.byref(s)), "sphx_get_stats")
        return s.as_dict()

    def reset_stats(self):
        self._check(self._lib.sphx_reset_stats(self._h), "sphx_reset_stats")

    def snapshot(self):
        self._check(self._lib.sphx_snapshot(self._h), "sphx_snapshot")

    def restore(self):
        self._check(self._lib.sphx_restore(self._h), "sphx_restore")

    def pairs_subset(self, sel) -> tuple[np.ndarray, np.ndarray]:
        """Neighbour lists of the particles `sel` (insertion indices) only."""
        sel = np.ascontiguousarray(sel, np.int64)
        counts = np.zeros(sel.size, np.int64)
        total = C.c_size_t(0)
        f = self._lib.sphx_debug_pairs_subset
        self._check(f(self._h, sel.size, _ptr(sel), _ptr(counts), None, C.byref(total)),
                    "sphx_debug_pairs_subset")
        idx = np.zeros(max(total.value, 1), np.int64)
        total2 = C.c_size_t(total.value)
        self._check(f(self._h, sel.size, _ptr(sel), _ptr(counts), _ptr(idx), C.byref(total2)),
                    "sphx_debug_pairs_subset")
        return counts, idx[: total2.value]

    def pairs(self) -> tuple[np.ndarray, np.ndarray]:
        """Neighbour lists of the current state: (counts[n], concatenated insertion ids)."""
        n = self.size()
        counts = np.zeros(n, np.int64)
        total = C.c_size_t(0)
        self._check(self._lib.sphx_debug_pairs(self._h, _ptr(counts), None, C.byref(total)),
                    "sphx_debug_pairs")
        idx = np.zeros(max(total.value, 1), np.int64)
        total2 = C.c_size_t(total.value)
        self._check(self._lib.sphx_debug_pairs(self._h, _ptr(counts), _ptr(idx),
                                               C.byref(total2)), "sphx_debug_pairs")
        return counts, idx[: total2.value]


def density_noalloc(params16, n: int, pos_ptr: int, mass_ptr: int, rho_ptr: int | None,
                    pressure_ptr: int | None, stream_ptr: int | None = None) -> None:
    """sphx_density_noalloc on caller-owned DEVICE buffers (raw pointers); asynchronous on
    the given stream."""
    cv = lambda p: C.c_void_p(p) if p else None
    rc = lib().sphx_density_noalloc(C.byref(params_struct(params16)), n, cv(pos_ptr),
                                    cv(mass_ptr), cv(rho_ptr), cv(pressure_ptr),
                                    cv(stream_ptr))
    if rc != OK:
        raise SphxError(rc, "sphx_density_noalloc")


class Grid:
    """Standalone GPU spatial hash (sphx_grid_*): SpatialHash build / query_squared."""

    def __init__(self, capacity: int):
        self._lib = lib()
        self._h = C.c_void_p()
        rc = self._lib.sphx_grid_create(C.byref(self._h), capacity)
        if rc != OK:
            raise SphxError(rc, "sphx_grid_create")

    def close(self):
        if self._h:
            self._lib.sphx_grid_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, where):
        if rc != OK:
            raise SphxError(rc, where)

    def build(self, pos, cell_size: float):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        self._check(self._lib.sphx_grid_build(self._h, pos.shape[0], _ptr(pos), C.c_float(cell_size)),
                    "sphx_grid_build")

    def query(self, q, radius_squared: float):
        q = np.ascontiguousarray(q, np.float32).reshape(-1, 3)
        nq = q.shape[0]
        counts = np.zeros(nq, np.int64)
        total = C.c_size_t(0)
        self._check(self._lib.sphx_grid_query(self._h, nq, _ptr(q), C.c_float(radius_squared),
                                               _ptr(counts), None, C.byref(total)), "sphx_grid_query")
        idx = np.zeros(max(total.value, 1), np.int64)
        t2 = C.c_size_t(total.value)
        self._check(self._lib.sphx_grid_query(self._h, nq, _ptr(q), C.c_float(radius_squared),
                                               _ptr(counts), _ptr(idx), C.byref(t2)), "sphx_grid_query")
        return counts, idx[: t2.value]

    def info(self):
        a, b = C.c_size_t(), C.c_size_t()
        self._check(self._lib.sphx_grid_info(self._h, C.byref(a), C.byref(b)), "sphx_grid_info")
        return a.value, b.value

    def cell(self, x: int, y: int, z: int):
        cnt = C.c_size_t(0)
        self._check(self._lib.sphx_grid_cell(self._h, x, y, z, None, C.byref(cnt)), "sphx_grid_cell")
        out = np.zeros(max(cnt.value, 1), np.int64)
        c2 = C.c_size_t(cnt.value)
        self._check(self._lib.sphx_grid_cell(self._h, x, y, z, _ptr(out), C.byref(c2)), "sphx_grid_cell")
        return out[: c2.value]
