"""GB300-native per-timestep boid update (drop-in for maru-n/BoidsSimulatorMPI).

The compute lives in ``libboids_gb300.so`` (hand-written sm_103a kernels
behind the C ABI of ``include/boids.h``).  This module binds that ABI with
ctypes and mirrors the reference's ``BoidSimulation`` interface
(src/boid_simulation.h:15-71): ``setup`` / ``init`` / ``update`` / ``get`` /
``get_v`` / ``get_force``, plus bulk accessors.  There is no CPU fallback:
importing the bindings fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libboids_gb300.so")

ENGINE_ALLPAIRS = 0
ENGINE_GRID = 1
FLAG_RECORD_FORCES = 1
FLAG_ALLPAIRS_KERNELS = 2

ERRORS = {-1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "EIO", -5: "ESTATE", -6: "ENOTSUP"}


class BoidsError(RuntimeError):
    """A negative status from the C ABI; ``code`` is the status."""

    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class Params(C.Structure):
    _fields_ = [("number_of_agents", C.c_uint32), ("field_size", C.c_double),
                ("separation_sight_distance", C.c_double), ("separation_sight_angle", C.c_double),
                ("separation_force_coefficient", C.c_double),
                ("alignment_sight_distance", C.c_double), ("alignment_sight_angle", C.c_double),
                ("alignment_force_coefficient", C.c_double),
                ("cohesion_sight_distance", C.c_double), ("cohesion_sight_angle", C.c_double),
                ("cohesion_force_coefficient", C.c_double),
                ("velocity_max", C.c_double), ("velocity_min", C.c_double),
                ("engine", C.c_int32), ("device", C.c_int32), ("flags", C.c_uint32),
                ("reserved", C.c_uint32)]


class GridInfo(C.Structure):
    _fields_ = [("ref_interaction_range", C.c_float), ("ref_grid_num", C.c_int32),
                ("ref_grid_size", C.c_float), ("dev_cells_per_axis", C.c_int32),
                ("dev_cell_size", C.c_float), ("list_capacity", C.c_int32)]


class Profile(C.Structure):
    _fields_ = [("bin_ms", C.c_double), ("force_ms", C.c_double), ("other_ms", C.c_double),
                ("steps", C.c_uint64), ("force_launches", C.c_uint64), ("bin_launches", C.c_uint64)]


# Every symbol include/boids.h declares, with its ctypes signature.
_vp = C.c_void_p
SIGNATURES = {
    "boids_create": (C.c_int, [C.POINTER(Params), C.POINTER(_vp)]),
    "boids_destroy": (None, [_vp]),
    "boids_init": (C.c_int, [_vp, C.c_char_p, C.c_int32]),
    "boids_init_ex": (C.c_int, [_vp, C.c_char_p, C.c_int32, C.c_int32]),
    "boids_set_state": (C.c_int, [_vp, _vp, _vp]),
    "boids_set_population": (C.c_int, [_vp, C.c_uint32, _vp, _vp]),
    "boids_step": (C.c_int, [_vp, C.c_int32]),
    "boids_get_state": (C.c_int, [_vp, _vp, _vp]),
    "boids_get_forces": (C.c_int, [_vp, _vp]),
    "boids_get_cells": (C.c_int, [_vp, _vp]),
    "boids_get_neighbor_sets": (C.c_int, [_vp, _vp, _vp]),
    "boids_get_grid_info": (C.c_int, [_vp, C.POINTER(GridInfo)]),
    "boids_set_stream": (C.c_int, [_vp, _vp]),
    "boids_synchronize": (C.c_int, [_vp]),
    "boids_profile_enable": (C.c_int, [_vp, C.c_int32]),
    "boids_profile_read": (C.c_int, [_vp, C.POINTER(Profile), C.c_int32]),
    "boids_kernel_launches": (C.c_uint64, [_vp]),
    "boids_set_tuning": (C.c_int, [_vp, _vp]),
    "boids_get_tuning": (C.c_int, [_vp, _vp]),
    "boids_autotune": (C.c_int, [_vp, C.c_int32]),
    "boids_frame_async": (C.c_int, [_vp, _vp, _vp, C.c_int32, C.c_int32]),
    "boids_frame_wait": (C.c_int, [_vp, C.c_int32]),
    "boids_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_vp)]),
    "boids_host_free": (None, [_vp]),
    "boids_ensemble_create": (C.c_int, [_vp, C.c_uint32, C.POINTER(_vp)]),
    "boids_ensemble_destroy": (None, [_vp]),
    "boids_ensemble_init": (C.c_int, [_vp]),
    "boids_ensemble_set_state": (C.c_int, [_vp, C.c_uint32, _vp, _vp]),
    "boids_ensemble_step": (C.c_int, [_vp, C.c_int32]),
    "boids_ensemble_get_state": (C.c_int, [_vp, C.c_uint32, _vp, _vp]),
    "boids_ensemble_stats": (C.c_int, [_vp, _vp]),
    "boids_ensemble_autotune": (C.c_int, [_vp, C.c_int32]),
    "boids_ensemble_tuning": (C.c_int, [_vp, _vp]),
    "boids_ensemble_set_tuning": (C.c_int, [_vp, _vp]),
    "boids_ensemble_synchronize": (C.c_int, [_vp]),
    "boids_ensemble_kernel_launches": (C.c_uint64, [_vp]),
    "boids_mlp_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_int32, C.POINTER(_vp)]),
    "boids_mlp_destroy": (None, [_vp]),
    "boids_mlp_param_count": (C.c_int64, [_vp]),
    "boids_mlp_get_params": (C.c_int, [_vp, _vp]),
    "boids_mlp_set_params": (C.c_int, [_vp, _vp]),
    "boids_mlp_forward": (C.c_int, [_vp, _vp, C.c_int32, _vp]),
    "boids_mlp_gradient": (C.c_int, [_vp, _vp, _vp, C.c_int32, _vp, C.POINTER(C.c_double)]),
    "boids_mlp_train": (C.c_int, [_vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                  C.POINTER(C.c_double)]),
    "boids_step_noalloc": (C.c_int, [C.POINTER(Params), _vp, _vp, _vp, _vp, _vp]),
    "boids_last_error": (C.c_char_p, []),
    "boids_version": (C.c_char_p, []),
}

_lib = None


def lib():
    """Loads libboids_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libboids_gb300.so is not built: run "
                               "`python -c 'import __graft_entry__ as g; g.build()'` or "
                               "`python boidssimulatormpi_gb300/build.py`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise BoidsError(rc, lib().boids_last_error().decode())


def _f32(a, n):
    a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    if a.size != n:
        raise ValueError("expected %d floats, got %d" % (n, a.size))
    return a


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class BoidSimulation:
    """Mirror of the reference's BoidSimulation over the C ABI.

    ``engine`` picks the link-time variant the reference has: "grid"
    (boidsim_grid, src/boid_simulation_grid.cpp) or "allpairs" (boidsim,
    src/boid_simulation.cpp).  The all-pairs engine runs the grid kernels
    where they fit (bit-identical results); ``allpairs_kernels=True`` keeps
    it on its own N^2 kernels.
    """

    def __init__(self, engine: str = "grid", device: int = 0, record_forces: bool = False,
                 allpairs_kernels: bool = False):
        self.engine = {"grid": ENGINE_GRID, "allpairs": ENGINE_ALLPAIRS}[engine]
        self.device = device
        self.record_forces = record_forces
        self.allpairs_kernels = allpairs_kernels
        self.h = None
        self.N = 0          # number_of_agents: the handle's capacity
        self.n_active = 0   # the population the getters cover (N, or set_population's n)
        self._cache = None

    # -- BoidSimulation::setup (src/boid_simulation.h:19-33)
    def setup(self, number_of_agents, field_size,
              separation_sight_distance, separation_sight_angle, separation_force_coefficient,
              alignment_sight_distance, alignment_sight_angle, alignment_force_coefficient,
              cohesion_sight_distance, cohesion_sight_angle, cohesion_force_coefficient,
              velocity_max, velocity_min, initialization="random_uniform", rand_seed=12345):
        self.close()
        p = Params(number_of_agents, field_size,
                   separation_sight_distance, separation_sight_angle, separation_force_coefficient,
                   alignment_sight_distance, alignment_sight_angle, alignment_force_coefficient,
                   cohesion_sight_distance, cohesion_sight_angle, cohesion_force_coefficient,
                   velocity_max, velocity_min, self.engine, self.device,
                   (FLAG_RECORD_FORCES if self.record_forces else 0)
                   | (FLAG_ALLPAIRS_KERNELS if self.allpairs_kernels else 0), 0)
        h = C.c_void_p()
        _check(lib().boids_create(C.byref(p), C.byref(h)))
        self.h = h
        self.params = p
        self.N = self.n_active = number_of_agents
        self.field_size_X = self.field_size_Y = self.field_size_Z = float(field_size)
        self.initialization_type = initialization
        self.rand_seed = rand_seed
        self.time_step = 0
        return self

    # -- BoidSimulation::init
    def init(self, seed_mode: int = -1):
        _check(lib().boids_init_ex(self.h, self.initialization_type.encode(), self.rand_seed, seed_mode))
        self.n_active = self.N
        self._cache = None

    # -- BoidSimulation::update
    def update(self, steps: int = 1):
        _check(lib().boids_step(self.h, steps))
        self._cache = None

    step = update

    def set_state(self, pos, vel):
        pos, vel = _f32(pos, 3 * self.N), _f32(vel, 3 * self.N)
        _check(lib().boids_set_state(self.h, _ptr(pos), _ptr(vel)))
        self.n_active = self.N
        self._cache = None

    def set_population(self, pos, vel):
        """The state of the first n boids, n = len(pos) // 3 (at most N)."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1)
        if pos.size % 3 or vel.size != pos.size:
            raise ValueError("positions and velocities must both hold 3 floats per boid")
        _check(lib().boids_set_population(self.h, pos.size // 3, _ptr(pos), _ptr(vel)))
        self.n_active = pos.size // 3
        self._cache = None

    def state(self, pos_out=None, vel_out=None):
        """(pos, vel) as float32 arrays of shape (n, 3), id order: n = N, or
        the population last set by set_population."""
        n = self.n_active
        pos = np.empty(3 * n, np.float32) if pos_out is None else pos_out
        vel = np.empty(3 * n, np.float32) if vel_out is None else vel_out
        _check(lib().boids_get_state(self.h, _ptr(pos), _ptr(vel)))
        return pos.reshape(n, 3), vel.reshape(n, 3)

    def positions(self, out=None):
        n = self.n_active
        pos = np.empty(3 * n, np.float32) if out is None else out
        _check(lib().boids_get_state(self.h, _ptr(pos), None))
        return pos.reshape(n, 3)

    def forces(self):
        """get_force for all ids: (n, 9) = cohesion xyz, separation xyz, alignment xyz."""
        n = self.n_active
        f = np.empty(9 * n, np.float32)
        _check(lib().boids_get_forces(self.h, _ptr(f)))
        return f.reshape(n, 9)

    def cells(self):
        """Boid::grid_index[8] of every boid, (n, 8) int32."""
        n = self.n_active
        g = np.empty(8 * n, np.int32)
        _check(lib().boids_get_cells(self.h, _ptr(g)))
        return g.reshape(n, 8)

    def neighbor_sets(self):
        """(count, hash), each (n, 3): per rule (cohesion, separation, alignment)."""
        n = self.n_active
        c = np.empty(3 * n, np.int32)
        h = np.empty(3 * n, np.uint64)
        _check(lib().boids_get_neighbor_sets(self.h, _ptr(c), _ptr(h)))
        return c.reshape(n, 3), h.reshape(n, 3)

    def grid_info(self) -> dict:
        gi = GridInfo()
        _check(lib().boids_get_grid_info(self.h, C.byref(gi)))
        return {f: getattr(gi, f) for f, _ in GridInfo._fields_}

    def set_stream(self, stream_handle: int | None):
        _check(lib().boids_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self):
        _check(lib().boids_synchronize(self.h))

    def profile_enable(self, on=True):
        _check(lib().boids_profile_enable(self.h, int(on)))

    def profile_read(self, reset=True) -> dict:
        pr = Profile()
        _check(lib().boids_profile_read(self.h, C.byref(pr), int(reset)))
        return {f: getattr(pr, f) for f, _ in Profile._fields_}

    def kernel_launches(self) -> int:
        return int(lib().boids_kernel_launches(self.h))

    # -- per-id getters of the reference (src/boid_simulation.h:37-43)
    def _state_cached(self):
        if self._cache is None:
            self._cache = self.state()
        return self._cache

    def get(self, i):
        p, _ = self._state_cached()
        return tuple(float(x) for x in p[i])

    def get_v(self, i):
        _, v = self._state_cached()
        return tuple(float(x) for x in v[i])

    def set_tuning(self, dense_min, defer_min, cand_defer, lone_cand):
        t = np.array([dense_min, defer_min, cand_defer, lone_cand], np.int32)
        _check(lib().boids_set_tuning(self.h, _ptr(t)))

    def tuning(self):
        t = np.zeros(4, np.int32)
        _check(lib().boids_get_tuning(self.h, _ptr(t)))
        return tuple(int(x) for x in t)

    def autotune(self, steps_per_trial=0):
        _check(lib().boids_autotune(self.h, steps_per_trial))
        self._cache = None
        return self.tuning()

    def get_force(self, i):
        return tuple(float(x) for x in self.forces()[i])

    def close(self):
        if self.h is not None and _lib is not None:
            _lib.boids_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def version() -> str:
    return lib().boids_version().decode()


# ------------------------------------------------------------------ ensembles

INIT_RANDOM_UNIFORM = 0
INIT_TEST = 1
STAT_NAMES = ("polarization", "milling", "nn_distance", "largest_cluster", "com_x", "com_y", "com_z",
              "momentum_x", "momentum_y", "momentum_z", "search_radius")


class FlockDesc(C.Structure):
    _fields_ = [("params", Params), ("init_kind", C.c_int32), ("rand_seed", C.c_int32)]


def flock_params(n, field, sep, ali, coh, vmax, vmin, device=0):
    """Params of one grid-engine flock; sep/ali/coh are (distance, angle, coefficient)."""
    return Params(n, field, *sep, *ali, *coh, vmax, vmin, ENGINE_GRID, device, 0, 0)


class Ensemble:
    """Many independent grid-engine flocks stepped together (boids_ensemble_*).

    ``flocks`` is a list of (Params, init_kind, rand_seed).  Each flock's
    trajectory is bit-identical to a BoidSimulation("grid") with the same
    parameters and seed."""

    def __init__(self, flocks):
        arr = (FlockDesc * len(flocks))()
        for i, (p, kind, seed) in enumerate(flocks):
            arr[i] = FlockDesc(p, kind, seed)
        h = C.c_void_p()
        _check(lib().boids_ensemble_create(C.cast(arr, C.c_void_p), len(flocks), C.byref(h)))
        self.h = h
        self.sizes = [p.number_of_agents for p, _, _ in flocks]

    def init(self):
        _check(lib().boids_ensemble_init(self.h))

    def step(self, steps=1):
        _check(lib().boids_ensemble_step(self.h, steps))

    def synchronize(self):
        _check(lib().boids_ensemble_synchronize(self.h))

    def set_state(self, flock, pos, vel):
        n = self.sizes[flock]
        p, v = _f32(pos, 3 * n), _f32(vel, 3 * n)
        _check(lib().boids_ensemble_set_state(self.h, flock, _ptr(p), _ptr(v)))

    def state(self, flock):
        n = self.sizes[flock]
        p = np.empty(3 * n, np.float32)
        v = np.empty(3 * n, np.float32)
        _check(lib().boids_ensemble_get_state(self.h, flock, _ptr(p), _ptr(v)))
        return p.reshape(n, 3), v.reshape(n, 3)

    def stats(self):
        out = np.empty((len(self.sizes), len(STAT_NAMES)), np.float64)
        _check(lib().boids_ensemble_stats(self.h, _ptr(out)))
        return out

    def autotune(self, steps_per_trial=0):
        _check(lib().boids_ensemble_autotune(self.h, steps_per_trial))
        return self.tuning()

    def tuning(self):
        t = np.zeros(4, np.int32)
        _check(lib().boids_ensemble_tuning(self.h, _ptr(t)))
        return tuple(int(x) for x in t)

    def set_tuning(self, dense_min, defer_min, cand_defer, lone_cand):
        t = np.array([min(int(x), 0x7fffffff) for x in (dense_min, defer_min, cand_defer, lone_cand)], np.int32)
        _check(lib().boids_ensemble_set_tuning(self.h, _ptr(t)))

    def kernel_launches(self):
        return int(lib().boids_ensemble_kernel_launches(self.h))

    def close(self):
        if self.h is not None and _lib is not None:
            _lib.boids_ensemble_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ sweep surrogate

class Surrogate:
    """The BF16 tensor-core MLP of boids_mlp_* (in -> hidden -> hidden -> out)."""

    def __init__(self, n_in=8, n_hidden=256, n_out=4, seed=1, device=0):
        h = C.c_void_p()
        _check(lib().boids_mlp_create(n_in, n_hidden, n_out, seed, device, C.byref(h)))
        self.h = h
        self.n_in, self.n_hidden, self.n_out = n_in, n_hidden, n_out

    def param_count(self):
        return int(lib().boids_mlp_param_count(self.h))

    def params(self):
        p = np.empty(self.param_count(), np.float32)
        _check(lib().boids_mlp_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = _f32(p, self.param_count())
        _check(lib().boids_mlp_set_params(self.h, _ptr(p)))

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.n_in)
        y = np.empty((x.shape[0], self.n_out), np.float32)
        _check(lib().boids_mlp_forward(self.h, _ptr(x), x.shape[0], _ptr(y)))
        return y

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.n_in)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, self.n_out)
        g = np.empty(self.param_count(), np.float32)
        loss = C.c_double()
        _check(lib().boids_mlp_gradient(self.h, _ptr(x), _ptr(t), x.shape[0], _ptr(g), C.byref(loss)))
        return g, loss.value

    def train(self, x, t, epochs=200, batch=256, lr=1e-3, seed=7):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.n_in)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, self.n_out)
        loss = C.c_double()
        _check(lib().boids_mlp_train(self.h, _ptr(x), _ptr(t), x.shape[0], epochs, batch, lr, seed,
                                     C.byref(loss)))
        return loss.value

    def close(self):
        if self.h is not None and _lib is not None:
            _lib.boids_mlp_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
