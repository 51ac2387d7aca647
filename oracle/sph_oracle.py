"""Python access to the oracle libraries.

TEST INFRASTRUCTURE ONLY.  Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm -- as the checker or the timed CPU baseline, never as part of the
product path.

  Port  -- oracle/_build/libsph_oracle.so, the C restatement (builds everywhere)
  Ref   -- oracle/_ref/libsph_ref.so, the reference's own sources compiled here
           (absent on machines without the reference checkout)
Both expose the same calls; Port has to agree with Ref bit for bit.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_PATH = HERE / "_build" / "libsph_oracle.so"
REF_PATH = HERE / "_ref" / "libsph_ref.so"
REF_FASTMATH_PATH = HERE / "_ref" / "libsph_ref_fastmath.so"


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class _Lib:
    prefix = ""

    def __init__(self, path: Path):
        if not path.exists():
            raise FileNotFoundError(path)
        self.path = path
        self.lib = C.CDLL(str(path))
        L, pf = self.lib, self.prefix
        q = getattr(L, f"{pf}_query")
        q.restype = C.c_int64
        q.argtypes = [C.c_size_t, C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p]
        f = getattr(L, f"{pf}_fields")
        f.restype = None
        f.argtypes = [C.c_size_t] + [C.c_void_p] * 7
        fk = getattr(L, f"{pf}_fields_k")
        fk.restype = None
        fk.argtypes = [C.c_int, C.c_size_t] + [C.c_void_p] * 7
        e = f"{pf}_engine_"
        getattr(L, e + "new").restype = C.c_void_p
        getattr(L, e + "new").argtypes = [C.c_size_t]
        for name in ("free", "clear"):
            getattr(L, e + name).argtypes = [C.c_void_p]
        getattr(L, e + "initialize").argtypes = [C.c_void_p, C.c_void_p]
        getattr(L, e + "add").argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p]
        getattr(L, e + "step").argtypes = [C.c_void_p, C.c_float]
        getattr(L, e + "size").restype = C.c_size_t
        getattr(L, e + "size").argtypes = [C.c_void_p]
        getattr(L, e + "time").restype = C.c_float
        getattr(L, e + "time").argtypes = [C.c_void_p]
        getattr(L, e + "diag").argtypes = [C.c_void_p, C.c_void_p]

    def query(self, pos, radius: float, cell_size: float | None = None):
        """Neighbour lists (counts, concatenated ids) in the reference's order."""
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        cs = radius if cell_size is None else cell_size
        fn = getattr(self.lib, f"{self.prefix}_query")
        counts = np.zeros(n, np.int64)
        total = fn(n, _p(pos), C.c_float(cs), C.c_float(radius), _p(counts), None)
        idx = np.zeros(max(total, 1), np.int64)
        fn(n, _p(pos), C.c_float(cs), C.c_float(radius), _p(counts), _p(idx))
        return counts, idx[:total]

    def fields(self, pos, vel, mass, params16, kernel: int = 0):
        """rho, P, acc of one evaluation of the step's field phases with the smoothing
        kernel `kernel` (0 cubic spline, 1 Wendland C2, 2 Gaussian)."""
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = _f32(vel).reshape(n, 3)
        mass = _f32(mass).reshape(n)
        prm = _f32(params16).reshape(16)
        rho = np.zeros(n, np.float32)
        P = np.zeros(n, np.float32)
        acc = np.zeros((n, 3), np.float32)
        getattr(self.lib, f"{self.prefix}_fields_k")(int(kernel), n, _p(pos), _p(vel), _p(mass),
                                                      _p(prm), _p(rho), _p(P), _p(acc))
        return rho, P, acc


class Port(_Lib):
    prefix = "orc"

    def __init__(self, path: Path = PORT_PATH):
        super().__init__(path)
        L = self.lib
        L.orc_query_subset.restype = C.c_int64
        L.orc_query_subset.argtypes = [C.c_size_t, C.c_void_p, C.c_float, C.c_float, C.c_size_t,
                                       C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_fields_f64.argtypes = [C.c_size_t] + [C.c_void_p] * 8
        L.orc_fields_f64_k.argtypes = [C.c_int, C.c_size_t] + [C.c_void_p] * 8
        L.orc_engine_set_kernel.argtypes = [C.c_void_p, C.c_int]
        L.orc_fields_f64d.argtypes = [C.c_size_t] + [C.c_void_p] * 7
        L.orc_fields_f64d.restype = C.c_int64
        L.orc_fields_f64d_s.argtypes = [C.c_size_t] + [C.c_void_p] * 8
        L.orc_fields_f64d_s.restype = C.c_int64
        L.orc_engine_get.argtypes = [C.c_void_p] + [C.c_void_p] * 5
        L.orc_engine_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_engine_last_dt.restype = C.c_float
        L.orc_engine_last_dt.argtypes = [C.c_void_p]
        L.orc_engine_step_count.restype = C.c_uint64
        L.orc_engine_step_count.argtypes = [C.c_void_p]
        L.orc_max_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_render_instances.argtypes = [C.c_void_p, C.c_size_t] + [C.c_void_p] * 4
        L.orc_render_image.argtypes = [C.c_void_p, C.c_size_t] + [C.c_void_p] * 4

    def query_subset(self, pos, radius: float, sel, cell_size: float | None = None):
        """Neighbour lists (counts, concatenated ids) of the particles `sel` only, in the
        reference's order, among all particles of `pos`."""
        pos = _f32(pos).reshape(-1, 3)
        sel = np.ascontiguousarray(sel, np.int64)
        cs = radius if cell_size is None else cell_size
        fn = self.lib.orc_query_subset
        counts = np.zeros(sel.size, np.int64)
        total = fn(pos.shape[0], _p(pos), C.c_float(cs), C.c_float(radius), sel.size, _p(sel),
                   _p(counts), None)
        idx = np.zeros(max(total, 1), np.int64)
        fn(pos.shape[0], _p(pos), C.c_float(cs), C.c_float(radius), sel.size, _p(sel),
           _p(counts), _p(idx))
        return counts, idx[:total]

    def fields_f64(self, pos, vel, mass, params16, want_scale: bool = False, kernel: int = 0):
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = _f32(vel).reshape(n, 3)
        mass = _f32(mass).reshape(n)
        prm = _f32(params16).reshape(16)
        rho = np.zeros(n)
        P = np.zeros(n)
        acc = np.zeros((n, 3))
        scale = np.zeros((n, 3)) if want_scale else None
        self.lib.orc_fields_f64_k(int(kernel), n, _p(pos), _p(vel), _p(mass), _p(prm), _p(rho),
                                  _p(P), _p(acc), _p(scale))
        return (rho, P, acc, scale) if want_scale else (rho, P, acc)

    def fields_f64d(self, pos64, vel, mass, params16, want_scale: bool = False):
        """FP64 density, pressure, acceleration on FP64 positions (sets in FP64); with
        want_scale also the per-component sum of |term| / m of each acceleration."""
        pos64 = np.ascontiguousarray(pos64, np.float64).reshape(-1, 3)
        n = pos64.shape[0]
        vel = _f32(vel).reshape(n, 3)
        mass = _f32(mass).reshape(n)
        prm = _f32(params16).reshape(16)
        rho = np.zeros(n)
        P = np.zeros(n)
        acc = np.zeros((n, 3))
        scale = np.zeros((n, 3)) if want_scale else None
        pairs = self.lib.orc_fields_f64d_s(n, _p(pos64), _p(vel), _p(mass), _p(prm), _p(rho),
                                           _p(P), _p(acc), _p(scale))
        return (rho, P, acc, pairs, scale) if want_scale else (rho, P, acc, pairs)

    def render_instances(self, rp, pos, vel, colors=None):
        """(n, 20) float32: clip-space corners and colour of every particle.  rp is a
        sphx_render_params-layout ctypes structure."""
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = _f32(vel).reshape(n, 3)
        col = None if colors is None else _f32(colors).reshape(n, 3)
        out = np.zeros((n, 20), np.float32)
        self.lib.orc_render_instances(C.byref(rp), n, _p(pos), _p(vel), _p(col), _p(out))
        return out

    def render_image(self, rp, pos, vel, colors=None):
        """(height, width, 4) uint8 image, rows bottom-up."""
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = _f32(vel).reshape(n, 3)
        col = None if colors is None else _f32(colors).reshape(n, 3)
        img = np.zeros((rp.height, rp.width, 4), np.uint8)
        self.lib.orc_render_image(C.byref(rp), n, _p(pos), _p(vel), _p(col), _p(img))
        return img

    def threads(self) -> int:
        return self.lib.orc_max_threads()

    def set_threads(self, n: int):
        self.lib.orc_set_threads(n)


class Ref(_Lib):
    prefix = "ref"

    def __init__(self, path: Path = REF_PATH):
        super().__init__(path)
        L = self.lib
        L.ref_engine_get.restype = C.c_size_t
        L.ref_engine_get.argtypes = [C.c_void_p] + [C.c_void_p] * 4


def have_ref() -> bool:
    return REF_PATH.exists()


class Engine:
    """An oracle engine (SPHEngine restatement or the reference itself)."""

    def __init__(self, lib: _Lib, capacity: int):
        self.o = lib
        self.pf = f"{lib.prefix}_engine_"
        self.cap = capacity
        self.h = C.c_void_p(getattr(lib.lib, self.pf + "new")(capacity))

    def __del__(self):
        try:
            getattr(self.o.lib, self.pf + "free")(self.h)
        except Exception:
            pass

    def initialize(self, params16):
        self._prm = _f32(params16).reshape(16)
        getattr(self.o.lib, self.pf + "initialize")(self.h, _p(self._prm))

    def add(self, pos, vel, mass):
        pos = _f32(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = None if vel is None else _f32(vel).reshape(n, 3)
        mass = _f32(mass).reshape(n)
        getattr(self.o.lib, self.pf + "add")(self.h, n, _p(pos), _p(vel), _p(mass))

    def step(self, dt: float):
        getattr(self.o.lib, self.pf + "step")(self.h, C.c_float(dt))

    def size(self) -> int:
        return getattr(self.o.lib, self.pf + "size")(self.h)

    def time(self) -> float:
        return getattr(self.o.lib, self.pf + "time")(self.h)

    def get(self):
        n = self.size()
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        rho = np.zeros(self.cap, np.float32)
        P = np.zeros(self.cap, np.float32)
        if isinstance(self.o, Port):
            acc = np.zeros((n, 3), np.float32)
            self.o.lib.orc_engine_get(self.h, _p(pos), _p(vel), _p(acc), _p(rho), _p(P))
            return dict(pos=pos, vel=vel, acc=acc, rho=rho[:n], pressure=P[:n],
                        rho_cap=rho, pressure_cap=P)
        self.o.lib.ref_engine_get(self.h, _p(pos), _p(vel), _p(rho), _p(P))
        return dict(pos=pos, vel=vel, rho=rho[:n], pressure=P[:n], rho_cap=rho, pressure_cap=P)

    def set_kernel(self, kind: int):
        """Smoothing kernel of the oracle engine's step (0 cubic spline, 1 Wendland C2,
        2 Gaussian)."""
        assert isinstance(self.o, Port)
        self.o.lib.orc_engine_set_kernel(self.h, int(kind))

    def set_state(self, pos, vel):
        assert isinstance(self.o, Port)
        self._state = (_f32(pos), _f32(vel))
        self.o.lib.orc_engine_set_state(self.h, _p(self._state[0]), _p(self._state[1]))

    def diag(self) -> np.ndarray:
        d = np.zeros(6)
        getattr(self.o.lib, self.pf + "diag")(self.h, _p(d))
        return d

    def last_dt(self) -> float:
        assert isinstance(self.o, Port)
        return self.o.lib.orc_engine_last_dt(self.h)


def bits_equal(a, b) -> bool:
    """Bitwise equality of float arrays, with every NaN equal to every NaN."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def mismatch_report(a, b, name="") -> str:
    a = np.asarray(a, np.float32).ravel()
    b = np.asarray(b, np.float32).ravel()
    bad = ~((a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b)))
    k = np.flatnonzero(bad)
    if k.size == 0:
        return f"{name}: identical"
    i = k[0]
    return (f"{name}: {k.size} of {a.size} differ; first at {i}: {a[i]!r} vs {b[i]!r}; "
            f"max abs diff {np.nanmax(np.abs(a[k].astype(np.float64) - b[k])):.3e}")
