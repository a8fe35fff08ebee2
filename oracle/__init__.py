"""TEST INFRASTRUCTURE ONLY: the CPU oracle for the per-timestep boid update.

``liboracle`` is the plain-C restatement in ``boids_oracle.c`` (FP32
arithmetic of the reference, operation by operation, plus an FP64 variant).
``RefEngine`` drives the reference engine itself, compiled from its own
sources by ``build_ref.sh`` into ``oracle/_ref`` where those sources exist.
Only tests, ``__graft_entry__.smoke()`` and ``bench.py`` (CPU baseline and
reference arm) import this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
BUILD_REF = os.path.join(HERE, "build_ref.sh")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")

RULES = ("cohesion", "separation", "alignment")


class OrcParams(C.Structure):
    _fields_ = [("n", C.c_uint32), ("field", C.c_double),
                ("sep_r", C.c_double), ("sep_a", C.c_double), ("sep_c", C.c_double),
                ("ali_r", C.c_double), ("ali_a", C.c_double), ("ali_c", C.c_double),
                ("coh_r", C.c_double), ("coh_a", C.c_double), ("coh_c", C.c_double),
                ("vmax", C.c_double), ("vmin", C.c_double)]


def build(quiet: bool = True) -> str:
    """Compile boids_oracle.c into liboracle.so (no-op when up to date)."""
    src = os.path.join(HERE, "boids_oracle.c")
    hdr = os.path.join(HERE, "boids_oracle.h")
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(hdr)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def ref_root() -> str | None:
    """The reference checkout: $REF_ROOT, else the default location that the
    recipe build_ref.sh names.  None when that directory is absent (machines
    without the reference sources: there the tests that need them skip)."""
    root = os.environ.get("REF_ROOT")
    if not root:
        r = subprocess.run(["bash", BUILD_REF, "--root"], capture_output=True, text=True)
        root = r.stdout.strip() if r.returncode == 0 else ""
    return root if root and os.path.isdir(root) else None


def build_ref(src_dir: str | None = None) -> bool:
    """Build oracle/_ref from the reference sources if they are present."""
    if not src_dir:
        root = ref_root()
        src_dir = os.environ.get("REF_SRC") or (os.path.join(root, "src") if root else "")
    if not src_dir or not os.path.exists(os.path.join(src_dir, "boid_simulation_grid.cpp")):
        return False
    subprocess.run(["bash", BUILD_REF, src_dir], check=True, capture_output=True)
    return True


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER(OrcParams)
        L.orc_init.argtypes = [P, C.c_int, C.c_int, C.c_int, _f32p, _f32p]
        L.orc_step_allpairs.argtypes = [P, _f32p, _f32p, C.c_void_p, C.c_int]
        L.orc_grid_geometry.argtypes = [P, C.POINTER(C.c_float), C.POINTER(C.c_int),
                                        C.POINTER(C.c_float)]
        L.orc_grid_create.argtypes = [P]
        L.orc_grid_create.restype = C.c_void_p
        L.orc_grid_bin.argtypes = [C.c_void_p, _f32p]
        L.orc_grid_step.argtypes = [C.c_void_p, _f32p, _f32p, C.c_void_p, C.c_int]
        L.orc_grid_destroy.argtypes = [C.c_void_p]
        L.orc_ref_cells.argtypes = [P, _f32p, _i32p]
        L.orc_neighbor_sets.argtypes = [P, _f32p, _f32p, _i32p, _u64p, C.c_int]
        L.orc_neighbor_sets_ex.argtypes = [P, _f32p, _f32p, _i32p, _u64p, C.c_int, C.c_int]
        L.orc_forces_f64.argtypes = [P, _f32p, _f32p, _f64p, C.c_int]
        L.orc_id_hash.argtypes = [C.c_uint32]
        L.orc_id_hash.restype = C.c_uint64
        _lib = L
    return _lib


def params(n, field, sep, ali, coh, vmax, vmin) -> OrcParams:
    """sep/ali/coh are (sight_distance, sight_angle, force_coefficient)."""
    return OrcParams(n, field, *sep, *ali, *coh, vmax, vmin)


def _f9(n):
    return np.zeros(9 * n, np.float32)


def init_state(p: OrcParams, kind: str = "random_uniform", seeded: bool = True, seed: int = 12345):
    k = {"random_uniform": 0, "test": 1}[kind]
    pos = np.zeros(3 * p.n, np.float32)
    vel = np.zeros(3 * p.n, np.float32)
    if lib().orc_init(C.byref(p), k, int(seeded), seed, pos, vel) != 0:
        raise ValueError(kind)
    return pos, vel


def step_allpairs(p, pos, vel, steps=1, threads=0, forces=False):
    """Advances (pos, vel) in place; returns the last step's get_force array."""
    f9 = _f9(p.n) if forces else None
    for _ in range(steps):
        lib().orc_step_allpairs(C.byref(p), pos, vel,
                                f9.ctypes.data if f9 is not None else None, threads)
    return f9


class GridPort:
    """The reference's overlapping-cell-list engine, restated in C."""

    def __init__(self, p: OrcParams, pos):
        self.p = p
        self.h = lib().orc_grid_create(C.byref(p))
        if not self.h:
            raise ValueError("Invalid GRID_NUM")
        lib().orc_grid_bin(self.h, pos)

    def step(self, pos, vel, steps=1, threads=0, forces=False):
        f9 = _f9(self.p.n) if forces else None
        for _ in range(steps):
            lib().orc_grid_step(self.h, pos, vel, f9.ctypes.data if f9 is not None else None,
                                threads)
        return f9

    def close(self):
        if self.h:
            lib().orc_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def grid_geometry(p):
    R, G, GS = C.c_float(), C.c_int(), C.c_float()
    rc = lib().orc_grid_geometry(C.byref(p), C.byref(R), C.byref(G), C.byref(GS))
    return None if rc != 0 else (R.value, G.value, GS.value)


def ref_cells(p, pos):
    out = np.zeros(8 * p.n, np.int32)
    if lib().orc_ref_cells(C.byref(p), pos, out) != 0:
        raise ValueError("Invalid GRID_NUM")
    return out.reshape(p.n, 8)


def neighbor_sets(p, pos, vel, threads=0, bucketed=True):
    cnt = np.zeros(3 * p.n, np.int32)
    h = np.zeros(3 * p.n, np.uint64)
    lib().orc_neighbor_sets_ex(C.byref(p), pos, vel, cnt, h, threads, int(bucketed))
    return cnt.reshape(p.n, 3), h.reshape(p.n, 3)


def forces_f64(p, pos, vel, threads=0):
    out = np.zeros(9 * p.n, np.float64)
    lib().orc_forces_f64(C.byref(p), pos, vel, out, threads)
    return out.reshape(p.n, 9)


def id_hash(i: int) -> int:
    return int(lib().orc_id_hash(i))


# ---------------------------------------------------------------- reference engine

def ref_available(kind: str = "grid") -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_%s.so" % kind))


class RefEngine:
    """BoidSimulation from the reference's own sources (kind 'grid' or
    'allpairs'), through the ref_* shim of ref_driver.cpp.  lib_path names
    another build of that shim (the same driver linked against another
    BoidSimulation, e.g. the GB300 engine's C++ adapter)."""

    _libs: dict = {}

    def __init__(self, kind, p: OrcParams, init="random_uniform", seed=12345, lib_path=None):
        L = self._load(kind, lib_path)
        self.L, self.n = L, p.n
        self.h = L.ref_create(p.n, p.field, p.sep_r, p.sep_a, p.sep_c, p.ali_r, p.ali_a,
                              p.ali_c, p.coh_r, p.coh_a, p.coh_c, p.vmax, p.vmin,
                              init.encode(), seed)
        self.kind = kind

    @classmethod
    def _load(cls, kind, lib_path=None):
        key = lib_path or kind
        if key not in cls._libs:
            path = lib_path or os.path.join(REF_DIR, "libref_%s.so" % kind)
            if not os.path.exists(path):
                raise FileNotFoundError(path)
            L = C.CDLL(path)
            d = C.c_double
            L.ref_create.argtypes = [C.c_uint] + [d] * 12 + [C.c_char_p, C.c_int]
            L.ref_create.restype = C.c_void_p
            for name in ("ref_init", "ref_destroy"):
                getattr(L, name).argtypes = [C.c_void_p]
            L.ref_set_state.argtypes = [C.c_void_p, _f32p, _f32p]
            L.ref_update.argtypes = [C.c_void_p, C.c_int]
            L.ref_get_state.argtypes = [C.c_void_p, _f32p, _f32p]
            L.ref_get_force.argtypes = [C.c_void_p, _f32p]
            L.ref_get_grid_index.argtypes = [C.c_void_p, _i32p]
            L.ref_grid_num.argtypes = [C.c_void_p]
            cls._libs[key] = L
        return cls._libs[key]

    def init(self, fresh_drand48=False):
        """BoidSimulation::init.  fresh_drand48 resets glibc's drand48 state to
        that of a new process first (the all-pairs engine never seeds it)."""
        if fresh_drand48:
            libc = C.CDLL(None)
            libc.seed48.argtypes = [C.POINTER(C.c_ushort)]
            libc.seed48((C.c_ushort * 3)(0, 0, 0))
        self.L.ref_init(self.h)

    def set_state(self, pos, vel):
        self.L.ref_set_state(self.h, np.ascontiguousarray(pos, np.float32),
                             np.ascontiguousarray(vel, np.float32))

    def update(self, steps=1):
        self.L.ref_update(self.h, steps)

    def state(self):
        pos = np.zeros(3 * self.n, np.float32)
        vel = np.zeros(3 * self.n, np.float32)
        self.L.ref_get_state(self.h, pos, vel)
        return pos, vel

    def forces(self):
        f = np.zeros(9 * self.n, np.float32)
        self.L.ref_get_force(self.h, f)
        return f

    def grid_index(self):
        g = np.zeros(8 * self.n, np.int32)
        self.L.ref_get_grid_index(self.h, g)
        return g.reshape(self.n, 8)

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- settings used by tests

MARUN2019 = dict(sep=(0.01, 0.5, 0.002), ali=(0.05, 0.3333333333333333, 0.06),
                 coh=(0.05, 0.5, 0.008), vmax=0.005, vmin=0.001)
TEST_INI = dict(sep=(0.1, 0.9, 0.0001), ali=(0.1, 0.7, 0.1), coh=(0.1, 0.8, 0.1),
                vmax=0.003, vmin=0.001)
