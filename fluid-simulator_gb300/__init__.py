"""pbf103: GB300-native Position Based Fluids step behind the reference solver API.

Python host mirror of the reference interface (DusanCojic/Fluid-Simulator,
``class PBFSolver`` in include/pbf/pbf_solver.hpp:13-70 and
``SimulationParams`` in include/pbf/simulation_params.hpp:6-29) over the C ABI
declared in include/pbf103.h.  Method names follow the reference
(initialize, set_particles, set_spheres, set_boxes, set_planes, step, run,
copy_positions_to_host, copy_velocities_to_host); errors raise the Python
counterparts of the C++ exception types the reference throws.

All compute runs in libpbf103.so (hand-written sm_103a kernels).  There is no
CPU fallback: importing succeeds without a GPU, but every call that needs the
library raises if it is not built or cannot reach a CUDA device.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import Iterable, Optional, Sequence

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libpbf103.so")

# ---------------------------------------------------------------------------
# Exceptions (status codes of include/pbf103.h <-> reference exception types)
# ---------------------------------------------------------------------------


class PBFError(Exception):
    """Base class of every error raised by this package."""


class InvalidArgument(PBFError, ValueError):
    """std::invalid_argument."""


class LogicError(PBFError, RuntimeError):
    """std::logic_error: the solver is used before initialize()."""


class OutOfRange(PBFError, IndexError):
    """std::out_of_range."""


class LengthError(PBFError, ValueError):
    """std::length_error."""


class NeighborOverflowError(PBFError, OverflowError):
    """std::overflow_error: a neighbour count exceeded the list capacity."""


class SolverRuntimeError(PBFError, RuntimeError):
    """std::runtime_error: CUDA failure or non-converging collisions."""


PBF_OK = 0
_STATUS_EXC = {
    1: InvalidArgument,
    2: LogicError,
    3: OutOfRange,
    4: LengthError,
    5: NeighborOverflowError,
    6: SolverRuntimeError,
}

# ---------------------------------------------------------------------------
# ctypes mirror of include/pbf103.h
# ---------------------------------------------------------------------------


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class _Params(C.Structure):
    _fields_ = [
        ("dt", C.c_float), ("restDensity", C.c_float), ("particleMass", C.c_float),
        ("particleRadius", C.c_float), ("collisionRestitution", C.c_float),
        ("collisionFriction", C.c_float), ("smoothingRadius", C.c_float),
        ("lambdaEpsilon", C.c_float), ("solverIterations", C.c_int), ("substeps", C.c_int),
        ("gravity", Float3), ("scorrK", C.c_float), ("scorrN", C.c_int),
        ("scorrDeltaQ", C.c_float), ("xsphViscosity", C.c_float),
        ("vorticityStrength", C.c_float),
    ]


@dataclasses.dataclass
class SimulationParams:
    """include/pbf/simulation_params.hpp:6-29, field for field."""

    dt: float = 1.0 / 60.0
    restDensity: float = 1000.0
    particleMass: float = 1.0
    particleRadius: float = 0.025
    collisionRestitution: float = 0.0
    collisionFriction: float = 0.0
    smoothingRadius: float = 0.1
    lambdaEpsilon: float = 100.0
    solverIterations: int = 4
    substeps: int = 1
    gravity: Sequence[float] = (0.0, -9.8, 0.0)
    scorrK: float = 0.0
    scorrN: int = 0
    scorrDeltaQ: float = 0.0
    xsphViscosity: float = 0.0
    vorticityStrength: float = 0.0

    def to_struct(self) -> _Params:
        s = _Params()
        for name, _ in _Params._fields_:
            if name == "gravity":
                g = self.gravity
                s.gravity = Float3(float(g[0]), float(g[1]), float(g[2]))
            else:
                setattr(s, name, getattr(self, name))
        return s

    def as_dict(self) -> dict:
        d = dataclasses.asdict(self)
        d["gravity"] = tuple(float(v) for v in self.gravity)
        return d


class _Scene(C.Structure):
    _fields_ = [("count", C.c_size_t), ("minBounds", Float3), ("maxBounds", Float3),
                ("restDensity", C.c_float), ("particleMass", C.c_float),
                ("xsphViscosity", C.c_float)]


@dataclasses.dataclass
class Scene:
    """One scene of a batched solver (pbf_scene): its particle count,
    container bounds and the parameters that may differ between scenes."""

    count: int
    minBounds: Sequence[float]
    maxBounds: Sequence[float]
    restDensity: float
    particleMass: float
    xsphViscosity: float

    def to_struct(self) -> _Scene:
        return _Scene(int(self.count), Float3(*map(float, self.minBounds)),
                      Float3(*map(float, self.maxBounds)), float(self.restDensity),
                      float(self.particleMass), float(self.xsphViscosity))


_lib = None
_vp = C.c_void_p


def _declare(L):
    S = C.c_int
    F3 = Float3
    sz = C.c_size_t
    fl = C.c_float
    sig = {
        "pbf_version": ([], C.c_char_p),
        "pbf_global_last_error": ([], C.c_char_p),
        "pbf_solver_create": ([C.POINTER(_vp), C.c_int], S),
        "pbf_solver_destroy": ([_vp], None),
        "pbf_last_error": ([_vp], C.c_char_p),
        "pbf_initialize": ([_vp, sz, F3, F3, C.POINTER(_Params)], S),
        "pbf_initialize_ex": ([_vp, sz, F3, F3, C.POINTER(_Params), C.c_int], S),
        "pbf_initialize_compact": ([_vp, sz, F3, F3, C.POINTER(_Params), C.c_int, sz], S),
        "pbf_set_particles": ([_vp, _vp, _vp, sz], S),
        "pbf_set_particles_device": ([_vp, _vp, _vp, sz], S),
        "pbf_set_spheres": ([_vp, _vp, sz], S),
        "pbf_set_boxes": ([_vp, _vp, sz], S),
        "pbf_set_planes": ([_vp, _vp, sz], S),
        "pbf_step": ([_vp], S),
        "pbf_run": ([_vp, sz], S),
        "pbf_run_async": ([_vp, sz], S),
        "pbf_synchronize": ([_vp], S),
        "pbf_time_frames": ([_vp, sz, C.POINTER(C.c_float)], S),
        "pbf_kernels_per_frame": ([_vp, C.POINTER(C.c_int)], S),
        "pbf_profile_frame": ([_vp, _vp, _vp], S),
        "pbf_stage_count": ([], C.c_int),
        "pbf_stage_name": ([C.c_int], C.c_char_p),
        "pbf_copy_positions": ([_vp, _vp, sz], S),
        "pbf_copy_velocities": ([_vp, _vp, sz], S),
        "pbf_copy_positions_device": ([_vp, _vp, sz], S),
        "pbf_copy_velocities_device": ([_vp, _vp, sz], S),
        "pbf_particle_count": ([_vp], sz),
        "pbf_batch_initialize": ([_vp, C.POINTER(_Scene), C.c_int, C.POINTER(_Params), C.c_int],
                                 S),
        "pbf_batch_scene_count": ([_vp], C.c_int),
        "pbf_autotune": ([_vp, C.c_int], S),
        "pbf_block_sizes": ([_vp, C.POINTER(C.c_int), C.c_int], S),
        "pbf_walk_lanes": ([_vp, C.POINTER(C.c_int)], S),
        "pbf_sort_tile": ([_vp, C.POINTER(C.c_int)], S),
        "pbf_set_walk_lanes": ([_vp, C.c_int], S),
        "pbf_adjoint_create": ([C.POINTER(_vp), C.c_int], S),
        "pbf_adjoint_destroy": ([_vp], None),
        "pbf_adjoint_last_error": ([_vp], C.c_char_p),
        "pbf_adjoint_initialize": ([_vp, sz, F3, F3, C.POINTER(_Params), C.c_int, C.c_int], S),
        "pbf_adjoint_set_physics": ([_vp, C.c_float, C.c_float], S),
        "pbf_adjoint_set_spheres": ([_vp, _vp, sz], S),
        "pbf_adjoint_set_boxes": ([_vp, _vp, sz], S),
        "pbf_adjoint_set_planes": ([_vp, _vp, sz], S),
        "pbf_adjoint_forward": ([_vp, _vp, _vp, C.c_int, _vp, _vp], S),
        "pbf_adjoint_backward": ([_vp, _vp, _vp, _vp, _vp, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)], S),
        "pbf_set_stream": ([_vp, _vp], S),
        "pbf_density_error": ([_vp, C.POINTER(C.c_double), C.POINTER(C.c_double)], S),
        "pbf_copy_working_state": ([_vp, _vp, _vp, _vp, sz], S),
        "pbf_grid_dims": ([F3, F3, fl, _vp], S),
        "pbf_grid_build": ([_vp, sz, F3, F3, fl, _vp, _vp, _vp, _vp], S),
        "pbf_find_neighbors": ([_vp, sz, _vp, _vp, _vp, F3, fl, fl, _vp, _vp, C.c_int, sz, _vp], S),
        "pbf_compute_lambda": ([_vp, _vp, _vp, C.c_int, sz, sz, fl, fl, fl, fl, _vp], S),
        "pbf_compute_delta": ([_vp, _vp, _vp, C.c_int, _vp, sz, sz, fl, fl, fl, fl, C.c_int, fl,
                               _vp], S),
        "pbf_xsph": ([_vp, _vp, _vp, C.c_int, _vp, _vp, sz, sz, fl, fl], S),
        "pbf_vorticity": ([_vp, _vp, _vp, _vp, C.c_int, sz, sz, fl, _vp], S),
        "pbf_confinement": ([_vp, _vp, _vp, C.c_int, _vp, _vp, _vp, sz, sz, fl, fl, fl], S),
        "pbf_collide": ([_vp, sz, F3, F3, _vp, sz, _vp, sz, _vp, sz, fl], S),
        "pbf_collision_pass": ([_vp, sz, C.c_int, F3, F3, _vp, sz, _vp, sz, _vp, sz, fl,
                                C.POINTER(C.c_int)], S),
        "pbf_resolve_velocities": ([_vp, _vp, _vp, sz, F3, F3, _vp, sz, _vp, sz, _vp, sz, fl, fl,
                                    fl], S),
        "pbf_integrate": ([_vp, _vp, _vp, sz, fl, F3], S),
        "pbf_grid_build_static_scratch": ([_vp, sz, F3, F3, fl, _vp, _vp, _vp, _vp, _vp], S),
        "pbf_static_scratch_capacity": ([], sz),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res


def library_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = True):
    """Load libpbf103.so (building it with nvcc when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise SolverRuntimeError("libpbf103.so is not built: run __graft_entry__.build()")
        from importlib import util as _u
        spec = _u.spec_from_file_location("_pbf103_build", os.path.join(PKG_DIR, "build.py"))
        mod = _u.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = C.CDLL(LIB_PATH)
    _declare(L)
    _lib = L
    return L


def version() -> str:
    return load().pbf_version().decode()


def _raise_global(st: int):
    if st != PBF_OK:
        msg = load().pbf_global_last_error().decode()
        raise _STATUS_EXC.get(st, SolverRuntimeError)(msg)


def _f3(v) -> Float3:
    return Float3(float(v[0]), float(v[1]), float(v[2]))


def _f4_array(a, name: str) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != 4:
        raise InvalidArgument("%s must be an (n, 4) float32 array" % name)
    return a


def _ptr(a) -> Optional[int]:
    return None if a is None else a.ctypes.data


def _colliders(items, width: int) -> np.ndarray:
    arr = np.asarray(list(items), dtype=np.float32)
    if arr.size == 0:
        return np.zeros((0, width), np.float32)
    return np.ascontiguousarray(arr.reshape(-1, width))


def _flatten_collider(c) -> list:
    """Accept (x,y,z,r) / ((x,y,z), r) / ((x,y,z),(a,b,c)) forms."""
    out = []
    for part in c:
        if isinstance(part, (tuple, list, np.ndarray)):
            out.extend(float(v) for v in part)
        else:
            out.append(float(part))
    return out


# ---------------------------------------------------------------------------
# Solver
# ---------------------------------------------------------------------------


class PBFSolver:
    """The reference's PBFSolver (src/pbf/pbf_solver.cu) on a GB300.

    Positions and velocities are (n, 4) float32 arrays (x, y, z, w); ``w`` is
    a payload the solver carries unchanged.  Outputs come back in the order
    the particles were given, whatever spatial order the solver works in.
    """

    def __init__(self, device: int = -1):
        L = load()
        h = _vp()
        _raise_global(L.pbf_solver_create(C.byref(h), device))
        self._h = h
        self._L = L

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.pbf_solver_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st: int):
        if st != PBF_OK:
            msg = self._L.pbf_last_error(self._h).decode()
            raise _STATUS_EXC.get(st, SolverRuntimeError)(msg)

    @property
    def handle(self) -> int:
        return self._h.value

    # -- reference API -------------------------------------------------------
    def initialize(self, max_particles: int, min_bounds, max_bounds, params: SimulationParams,
                   max_neighbors: int = 256, list_capacity: Optional[int] = None):
        """PBFSolver::initialize.  list_capacity: compact neighbour lists of
        that many entries in all (pbf_initialize_compact) instead of
        max_neighbors slots per particle."""
        self._params = params.to_struct()
        if list_capacity is not None:
            st = self._L.pbf_initialize_compact(self._h, int(max_particles), _f3(min_bounds),
                                                _f3(max_bounds), C.byref(self._params),
                                                int(max_neighbors), int(list_capacity))
        elif max_neighbors == 256:
            st = self._L.pbf_initialize(self._h, int(max_particles), _f3(min_bounds),
                                        _f3(max_bounds), C.byref(self._params))
        else:
            st = self._L.pbf_initialize_ex(self._h, int(max_particles), _f3(min_bounds),
                                           _f3(max_bounds), C.byref(self._params),
                                           int(max_neighbors))
        self._check(st)

    def initialize_batch(self, scenes: Sequence[Scene], common: SimulationParams,
                         max_neighbors: int = 256):
        """pbf_batch_initialize: the scenes step together; particles are set
        and copied as the concatenation of all scenes in order."""
        self._params = common.to_struct()
        arr = (_Scene * len(scenes))(*[sc.to_struct() for sc in scenes])
        self._scenes = arr
        self._check(self._L.pbf_batch_initialize(self._h, arr, len(scenes),
                                                 C.byref(self._params), int(max_neighbors)))

    def scene_count(self) -> int:
        return int(self._L.pbf_batch_scene_count(self._h))

    TUNED_KERNELS = ("search_lambda", "delta_apply", "search_final", "xsph", "vorticity",
                     "confine")

    def autotune(self, frames_per_trial: int = 2) -> dict:
        """pbf_autotune: choose the neighbour kernels' block sizes and the sort
        tile; returns them."""
        self._check(self._L.pbf_autotune(self._h, int(frames_per_trial)))
        return self.block_sizes()

    def block_sizes(self) -> dict:
        """Threads per block of the six tuned kernels and the sort's keys per tile."""
        out = (C.c_int * 6)()
        self._check(self._L.pbf_block_sizes(self._h, out, 6))
        tile = C.c_int()
        self._check(self._L.pbf_sort_tile(self._h, C.byref(tile)))
        return dict(zip(self.TUNED_KERNELS, list(out)), sort_tile=tile.value)

    def walk_lanes(self) -> int:
        """Lanes per particle of the list-writing walks (pbf_walk_lanes)."""
        k = C.c_int()
        self._check(self._L.pbf_walk_lanes(self._h, C.byref(k)))
        return k.value

    def set_walk_lanes(self, lanes: int):
        """pbf_set_walk_lanes: 1, 2, 4 or 8 lanes per particle, 0 = default."""
        self._check(self._L.pbf_set_walk_lanes(self._h, int(lanes)))

    def set_particles(self, positions, velocities, count: Optional[int] = None):
        if positions is None or velocities is None:
            n = 0 if count is None else int(count)
            self._check(self._L.pbf_set_particles(self._h, None, None, n))
            return
        p = _f4_array(positions, "positions")
        v = _f4_array(velocities, "velocities")
        n = p.shape[0] if count is None else int(count)
        if n > p.shape[0] or n > v.shape[0]:
            raise OutOfRange("count exceeds the given arrays")
        self._check(self._L.pbf_set_particles(self._h, _ptr(p), _ptr(v), n))

    def set_particles_device(self, positions, velocities):
        """positions/velocities: contiguous float32 CUDA tensors of shape (n, 4)."""
        n = int(positions.shape[0])
        self._check(self._L.pbf_set_particles_device(self._h, positions.data_ptr(),
                                                     velocities.data_ptr(), n))

    def set_spheres(self, spheres: Iterable):
        arr = _colliders([_flatten_collider(s) for s in spheres], 4)
        self._check(self._L.pbf_set_spheres(self._h, _ptr(arr), arr.shape[0]))

    def set_boxes(self, boxes: Iterable):
        arr = _colliders([_flatten_collider(b) for b in boxes], 6)
        self._check(self._L.pbf_set_boxes(self._h, _ptr(arr), arr.shape[0]))

    def set_planes(self, planes: Iterable):
        arr = _colliders([_flatten_collider(p) for p in planes], 6)
        self._check(self._L.pbf_set_planes(self._h, _ptr(arr), arr.shape[0]))

    def step(self):
        self._check(self._L.pbf_step(self._h))

    def run(self, frames: Optional[int] = None):
        """run() advances one frame; run(n) advances n frames."""
        self._check(self._L.pbf_run(self._h, 1 if frames is None else int(frames)))

    def run_async(self, frames: int):
        self._check(self._L.pbf_run_async(self._h, int(frames)))

    def synchronize(self):
        self._check(self._L.pbf_synchronize(self._h))

    def time_frames(self, frames: int) -> float:
        ms = C.c_float()
        self._check(self._L.pbf_time_frames(self._h, int(frames), C.byref(ms)))
        return ms.value

    def kernels_per_frame(self) -> int:
        k = C.c_int()
        self._check(self._L.pbf_kernels_per_frame(self._h, C.byref(k)))
        return k.value

    def profile_frame(self) -> dict:
        """One frame with CUDA events between stages: {stage: (ms, launches)}."""
        k = self._L.pbf_stage_count()
        ms = np.zeros(k, np.float32)
        launches = np.zeros(k, np.int32)
        self._check(self._L.pbf_profile_frame(self._h, ms.ctypes.data, launches.ctypes.data))
        return {self._L.pbf_stage_name(i).decode(): (float(ms[i]), int(launches[i]))
                for i in range(k) if launches[i]}

    def set_stream(self, stream_handle: Optional[int]):
        self._check(self._L.pbf_set_stream(self._h, stream_handle))

    @property
    def particle_count(self) -> int:
        return int(self._L.pbf_particle_count(self._h))

    def copy_positions_to_host(self, count: Optional[int] = None, out=None) -> np.ndarray:
        n = self.particle_count if count is None else int(count)
        if out is None:
            out = np.zeros((max(n, 0), 4), np.float32)
        self._check(self._L.pbf_copy_positions(self._h, _ptr(out) if n else None, n))
        return out

    def copy_velocities_to_host(self, count: Optional[int] = None, out=None) -> np.ndarray:
        n = self.particle_count if count is None else int(count)
        if out is None:
            out = np.zeros((max(n, 0), 4), np.float32)
        self._check(self._L.pbf_copy_velocities(self._h, _ptr(out) if n else None, n))
        return out

    def copy_positions_raw(self, ptr, count: int):
        """copyPositionsToHost with a raw destination pointer (may be None)."""
        self._check(self._L.pbf_copy_positions(self._h, ptr, int(count)))

    def copy_velocities_raw(self, ptr, count: int):
        self._check(self._L.pbf_copy_velocities(self._h, ptr, int(count)))

    def copy_positions_device(self, out_tensor):
        self._check(self._L.pbf_copy_positions_device(self._h, out_tensor.data_ptr(),
                                                      int(out_tensor.shape[0])))

    def copy_velocities_device(self, out_tensor):
        self._check(self._L.pbf_copy_velocities_device(self._h, out_tensor.data_ptr(),
                                                       int(out_tensor.shape[0])))

    def density_error(self):
        m, x = C.c_double(), C.c_double()
        self._check(self._L.pbf_density_error(self._h, C.byref(m), C.byref(x)))
        return m.value, x.value

    def working_state(self):
        n = self.particle_count
        pos = np.zeros((n, 4), np.float32)
        ids = np.zeros(n, np.uint32)
        cnt = np.zeros(n, np.int32)
        self._check(self._L.pbf_copy_working_state(self._h, _ptr(pos), _ptr(ids), _ptr(cnt), n))
        return pos, ids, cnt


# ---------------------------------------------------------------------------
# Stage entry points (the reference's kernel-level API)
# ---------------------------------------------------------------------------


def grid_dims(min_bounds, max_bounds, cell_size):
    d = (C.c_int * 3)()
    _raise_global(load().pbf_grid_dims(_f3(min_bounds), _f3(max_bounds), float(cell_size), d))
    return (d[0], d[1], d[2])


def grid_build(positions, min_bounds, max_bounds, cell_size):
    """SpatialGrid::initialize + build: (sorted_keys, sorted_indices, cell_start, cell_end)."""
    dims = grid_dims(min_bounds, max_bounds, cell_size)
    cells = dims[0] * dims[1] * dims[2]
    p = _f4_array(positions, "positions") if len(positions) else np.zeros((0, 4), np.float32)
    n = p.shape[0]
    sk = np.zeros(n, np.uint32)
    si = np.zeros(n, np.uint32)
    cs = np.zeros(cells, np.int32)
    ce = np.zeros(cells, np.int32)
    _raise_global(load().pbf_grid_build(_ptr(p) if n else None, n, _f3(min_bounds),
                                        _f3(max_bounds), float(cell_size), _ptr(sk) if n else None,
                                        _ptr(si) if n else None, _ptr(cs), _ptr(ce)))
    return sk, si, cs, ce


def find_neighbors(sorted_positions, cell_start, cell_end, dims, min_bounds, cell_size,
                   smoothing_radius, max_neighbors=256, stride=None, fill=0xFFFFFFFF):
    """findNeighbors: (slot-major neighbours, counts, overflow flag)."""
    p = _f4_array(sorted_positions, "positions")
    n = p.shape[0]
    stride = n if stride is None else int(stride)
    nb = np.full(stride * max_neighbors, fill, np.uint32)
    cnt = np.zeros(n, np.int32)
    ov = C.c_int()
    d = (C.c_int * 3)(*dims)
    cs = np.ascontiguousarray(cell_start, np.int32)
    ce = np.ascontiguousarray(cell_end, np.int32)
    _raise_global(load().pbf_find_neighbors(_ptr(p), n, _ptr(cs), _ptr(ce), d, _f3(min_bounds),
                                            float(cell_size), float(smoothing_radius),
                                            _ptr(nb) if nb.size else None, _ptr(cnt),
                                            int(max_neighbors), stride, C.byref(ov)))
    return nb, cnt, bool(ov.value)


def compute_lambda(positions, neighbors, counts, max_neighbors, stride, h, mass, rho0, eps):
    p = _f4_array(positions, "positions")
    out = np.zeros(p.shape[0], np.float32)
    nb = np.ascontiguousarray(neighbors, np.uint32)
    cnt = np.ascontiguousarray(counts, np.int32)
    _raise_global(load().pbf_compute_lambda(_ptr(p), _ptr(nb), _ptr(cnt), int(max_neighbors),
                                            p.shape[0], int(stride), h, mass, rho0, eps,
                                            _ptr(out)))
    return out


def compute_delta(positions, neighbors, counts, max_neighbors, lambdas, stride, h, mass, rho0,
                  scorr_k, scorr_n, scorr_dq):
    p = _f4_array(positions, "positions")
    out = np.zeros_like(p)
    nb = np.ascontiguousarray(neighbors, np.uint32)
    cnt = np.ascontiguousarray(counts, np.int32)
    lam = np.ascontiguousarray(lambdas, np.float32)
    _raise_global(load().pbf_compute_delta(_ptr(p), _ptr(nb), _ptr(cnt), int(max_neighbors),
                                           _ptr(lam), p.shape[0], int(stride), h, mass, rho0,
                                           scorr_k, int(scorr_n), scorr_dq, _ptr(out)))
    return out


def xsph(positions, neighbors, counts, max_neighbors, velocities, stride, h, viscosity):
    p = _f4_array(positions, "positions")
    v = _f4_array(velocities, "velocities")
    out = np.zeros_like(v)
    nb = np.ascontiguousarray(neighbors, np.uint32)
    cnt = np.ascontiguousarray(counts, np.int32)
    _raise_global(load().pbf_xsph(_ptr(p), _ptr(nb), _ptr(cnt), int(max_neighbors), _ptr(v),
                                  _ptr(out), p.shape[0], int(stride), h, viscosity))
    return out


def vorticity(positions, velocities, neighbors, counts, max_neighbors, stride, h):
    p = _f4_array(positions, "positions")
    v = _f4_array(velocities, "velocities")
    out = np.zeros_like(v)
    nb = np.ascontiguousarray(neighbors, np.uint32)
    cnt = np.ascontiguousarray(counts, np.int32)
    _raise_global(load().pbf_vorticity(_ptr(p), _ptr(v), _ptr(nb), _ptr(cnt), int(max_neighbors),
                                       p.shape[0], int(stride), h, _ptr(out)))
    return out


def confinement(positions, neighbors, counts, max_neighbors, omega, velocities, stride, h, dt,
                strength):
    p = _f4_array(positions, "positions")
    om = _f4_array(omega, "omega")
    v = _f4_array(velocities, "velocities")
    out = np.zeros_like(v)
    nb = np.ascontiguousarray(neighbors, np.uint32)
    cnt = np.ascontiguousarray(counts, np.int32)
    _raise_global(load().pbf_confinement(_ptr(p), _ptr(nb), _ptr(cnt), int(max_neighbors),
                                         _ptr(om), _ptr(v), _ptr(out), p.shape[0], int(stride), h,
                                         dt, strength))
    return out


def _collider_arrays(spheres, boxes, planes):
    sp = _colliders([_flatten_collider(s) for s in spheres], 4)
    bx = _colliders([_flatten_collider(b) for b in boxes], 6)
    pl = _colliders([_flatten_collider(p) for p in planes], 6)
    return sp, bx, pl


def collision_pass(positions, kind, container_min, container_max, particle_radius, spheres=(),
                   boxes=(), planes=()):
    """One projection kernel: kind 0 container, 1 spheres, 2 boxes, 3 planes."""
    p = _f4_array(positions, "positions").copy()
    sp, bx, pl = _collider_arrays(spheres, boxes, planes)
    flag = C.c_int()
    _raise_global(load().pbf_collision_pass(
        _ptr(p) if p.shape[0] else None, p.shape[0], int(kind), _f3(container_min),
        _f3(container_max), _ptr(sp) if sp.shape[0] else None, sp.shape[0],
        _ptr(bx) if bx.shape[0] else None, bx.shape[0], _ptr(pl) if pl.shape[0] else None,
        pl.shape[0], float(particle_radius), C.byref(flag)))
    return p, bool(flag.value)


def collide(positions, container_min, container_max, particle_radius, spheres=(), boxes=(),
            planes=()):
    """CollisionSystem::solve; raises SolverRuntimeError when it does not converge."""
    p = _f4_array(positions, "positions").copy()
    sp, bx, pl = _collider_arrays(spheres, boxes, planes)
    _raise_global(load().pbf_collide(
        _ptr(p) if p.shape[0] else None, p.shape[0], _f3(container_min), _f3(container_max),
        _ptr(sp) if sp.shape[0] else None, sp.shape[0], _ptr(bx) if bx.shape[0] else None,
        bx.shape[0], _ptr(pl) if pl.shape[0] else None, pl.shape[0], float(particle_radius)))
    return p


def resolve_velocities(positions, incoming, velocities, container_min, container_max,
                       particle_radius, restitution, friction, spheres=(), boxes=(), planes=()):
    p = _f4_array(positions, "positions")
    vi = _f4_array(incoming, "incoming")
    v = _f4_array(velocities, "velocities").copy()
    sp, bx, pl = _collider_arrays(spheres, boxes, planes)
    _raise_global(load().pbf_resolve_velocities(
        _ptr(p), _ptr(vi), _ptr(v), p.shape[0], _f3(container_min), _f3(container_max),
        _ptr(sp) if sp.shape[0] else None, sp.shape[0], _ptr(bx) if bx.shape[0] else None,
        bx.shape[0], _ptr(pl) if pl.shape[0] else None, pl.shape[0], float(particle_radius),
        float(restitution), float(friction)))
    return v


def integrate(positions, velocities, dt, gravity):
    p = _f4_array(positions, "positions")
    v = _f4_array(velocities, "velocities").copy()
    xs = np.zeros_like(p)
    _raise_global(load().pbf_integrate(_ptr(p), _ptr(xs), _ptr(v), p.shape[0], float(dt),
                                       _f3(gravity)))
    return xs, v


class PBFAdjoint:
    """Reverse-mode derivative of ``steps`` solver steps (pbf_adjoint_*).

    ``forward`` runs the differentiated step (integration, density
    constraint with s_corr and the collision projection, velocity update,
    XSPH, vorticity confinement, velocity response) from (x0, v0),
    keeping checkpoints;
    ``backward`` takes dL/dx, dL/dv of that forward's final state and returns
    dL/dx0, dL/dv0, dL/drestDensity and dL/dxsphViscosity.  Arrays are (n, 4)
    float32 numpy arrays or contiguous CUDA tensors (anything with a
    ``data_ptr``); outputs come back in the same kind as ``x0``.
    """

    def __init__(self, device: int = -1):
        L = load()
        h = _vp()
        _raise_global(L.pbf_adjoint_create(C.byref(h), device))
        self._h = h
        self._L = L
        self.n = 0

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.pbf_adjoint_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != PBF_OK:
            msg = self._L.pbf_adjoint_last_error(self._h).decode()
            raise _STATUS_EXC.get(st, SolverRuntimeError)(msg)

    def initialize(self, count: int, min_bounds, max_bounds, params: SimulationParams,
                   max_neighbors: int = 128, checkpoint_every: int = 10):
        self._params = params.to_struct()
        self._check(self._L.pbf_adjoint_initialize(self._h, int(count), _f3(min_bounds),
                                                   _f3(max_bounds), C.byref(self._params),
                                                   int(max_neighbors), int(checkpoint_every)))
        self.n = int(count)

    def set_physics(self, rest_density: float, xsph_viscosity: float):
        self._check(self._L.pbf_adjoint_set_physics(self._h, float(rest_density),
                                                    float(xsph_viscosity)))

    def set_spheres(self, spheres: Iterable):
        """Sphere colliders of the differentiated step (drops the forward)."""
        arr = _colliders([_flatten_collider(c) for c in spheres], 4)
        self._check(self._L.pbf_adjoint_set_spheres(self._h, _ptr(arr), arr.shape[0]))

    def set_boxes(self, boxes: Iterable):
        arr = _colliders([_flatten_collider(c) for c in boxes], 6)
        self._check(self._L.pbf_adjoint_set_boxes(self._h, _ptr(arr), arr.shape[0]))

    def set_planes(self, planes: Iterable):
        arr = _colliders([_flatten_collider(c) for c in planes], 6)
        self._check(self._L.pbf_adjoint_set_planes(self._h, _ptr(arr), arr.shape[0]))

    @staticmethod
    def _arg(a, name, n):
        if hasattr(a, "data_ptr"):
            if tuple(a.shape) != (n, 4) or not a.is_contiguous():
                raise InvalidArgument("%s must be a contiguous (n, 4) tensor" % name)
            return a, a.data_ptr()
        a = _f4_array(a, name)
        if a.shape[0] != n:
            raise InvalidArgument("%s must have %d rows" % (name, n))
        return a, a.ctypes.data

    def _like(self, ref):
        if hasattr(ref, "data_ptr"):
            import torch
            t = torch.empty((self.n, 4), dtype=torch.float32, device=ref.device)
            return t, t.data_ptr()
        a = np.zeros((self.n, 4), np.float32)
        return a, a.ctypes.data

    def forward(self, x0, v0, steps: int):
        x0, px = self._arg(x0, "x0", self.n)
        v0, pv = self._arg(v0, "v0", self.n)
        xo, pxo = self._like(x0)
        vo, pvo = self._like(x0)
        self._check(self._L.pbf_adjoint_forward(self._h, px, pv, int(steps), pxo, pvo))
        return xo, vo

    def backward(self, grad_x, grad_v):
        gx, pgx = self._arg(grad_x, "grad_x", self.n)
        gv, pgv = self._arg(grad_v, "grad_v", self.n)
        gx0, p0 = self._like(gx)
        gv0, p1 = self._like(gx)
        gr, gc = C.c_double(), C.c_double()
        self._check(self._L.pbf_adjoint_backward(self._h, pgx, pgv, p0, p1, C.byref(gr),
                                                 C.byref(gc)))
        return gx0, gv0, gr.value, gc.value
