"""ctypes wrapper around the CPU oracle (pbf_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference solver step
(DusanCojic/Fluid-Simulator, src/pbf/pbf_solver.cu:186-328) on the host.  Only
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline arm may import
this module; the CUDA product never routes through it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpbf_oracle.so")
SRC = os.path.join(HERE, "pbf_oracle.cpp")
SOURCES = [SRC, os.path.join(HERE, "pbf_diff_oracle.cpp")]

ORC_OK, ORC_ERR_INVALID, ORC_ERR_LENGTH, ORC_ERR_OVERFLOW, ORC_ERR_NOT_CONVERGED = range(5)


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (OpenMP, no FP contraction)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = SOURCES + [os.path.join(HERE, "pbf_oracle.h")]
    if (not force and os.path.exists(LIB_PATH)
            and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d) for d in deps)):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp] + SOURCES
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class F3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Params(C.Structure):
    """Same field order as SimulationParams (include/pbf/simulation_params.hpp:6-29)."""
    _fields_ = [
        ("dt", C.c_float), ("restDensity", C.c_float), ("particleMass", C.c_float),
        ("particleRadius", C.c_float), ("collisionRestitution", C.c_float),
        ("collisionFriction", C.c_float), ("smoothingRadius", C.c_float),
        ("lambdaEpsilon", C.c_float), ("solverIterations", C.c_int), ("substeps", C.c_int),
        ("gravity", F3), ("scorrK", C.c_float), ("scorrN", C.c_int),
        ("scorrDeltaQ", C.c_float), ("xsphViscosity", C.c_float),
        ("vorticityStrength", C.c_float),
    ]


class Container(C.Structure):
    _fields_ = [("min", F3), ("max", F3)]


_lib = None
_fp = C.POINTER(C.c_float)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int)
_vp = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_diff_rollout.argtypes = [C.c_size_t, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int,
                                       _vp, F3, F3, C.c_int, _vp, _vp, _vp, _vp, _vp]
        L.orc_diff_rollout.restype = C.c_int
        L.orc_diff_rollout_phys.argtypes = L.orc_diff_rollout.argtypes + [_vp]
        L.orc_diff_rollout_phys.restype = C.c_int
        L.orc_diff_rollout_col.argtypes = L.orc_diff_rollout_phys.argtypes + [
            _vp, C.c_size_t, _vp, C.c_size_t, _vp, C.c_size_t]
        L.orc_diff_rollout_col.restype = C.c_int
        L.orc_grid_dims.argtypes = [F3, F3, C.c_float, _i32p]
        L.orc_grid_dims.restype = C.c_int
        L.orc_grid_build.argtypes = [_vp, C.c_size_t, F3, C.c_float, _i32p, _vp, _vp, _vp, _vp]
        L.orc_find_neighbors.argtypes = [_vp, C.c_size_t, _vp, _vp, _i32p, F3, C.c_float,
                                         C.c_float, _vp, _vp, C.c_int, C.c_size_t]
        L.orc_find_neighbors.restype = C.c_int
        L.orc_lambda.argtypes = [_vp, _vp, _vp, C.c_int, C.c_size_t, C.c_size_t, C.c_float,
                                 C.c_float, C.c_float, C.c_float, _vp]
        L.orc_delta.argtypes = [_vp, _vp, _vp, C.c_int, _vp, C.c_size_t, C.c_size_t,
                                C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                C.c_float, _vp]
        L.orc_scorr.argtypes = [C.c_float] * 4 + [C.c_int, C.c_float]
        L.orc_scorr.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.c_float]
        L.orc_scorr.restype = C.c_float
        L.orc_poly6.argtypes = [C.c_float, C.c_float]
        L.orc_poly6.restype = C.c_float
        L.orc_spiky.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, _fp]
        L.orc_xsph.argtypes = [_vp, _vp, _vp, C.c_int, _vp, _vp, C.c_size_t, C.c_size_t,
                               C.c_float, C.c_float]
        L.orc_vorticity.argtypes = [_vp, _vp, _vp, _vp, C.c_int, C.c_size_t, C.c_size_t,
                                    C.c_float, _vp]
        L.orc_confinement.argtypes = [_vp, _vp, _vp, C.c_int, _vp, _vp, _vp, C.c_size_t,
                                      C.c_size_t, C.c_float, C.c_float, C.c_float]
        L.orc_solve_container.argtypes = [_vp, C.c_size_t, Container, C.c_float]
        L.orc_solve_container.restype = C.c_int
        for nm in ("orc_solve_spheres", "orc_solve_boxes", "orc_solve_planes"):
            getattr(L, nm).argtypes = [_vp, C.c_size_t, _vp, C.c_size_t, C.c_float]
            getattr(L, nm).restype = C.c_int
        L.orc_collide.argtypes = [_vp, C.c_size_t, Container, _vp, C.c_size_t, _vp,
                                  C.c_size_t, _vp, C.c_size_t, C.c_float, C.c_int]
        L.orc_collide.restype = C.c_int
        L.orc_resolve_velocities.argtypes = [_vp, _vp, _vp, C.c_size_t, Container, _vp,
                                             C.c_size_t, _vp, C.c_size_t, _vp, C.c_size_t,
                                             C.c_float, C.c_float, C.c_float]
        L.orc_solver_create.argtypes = [C.c_int]
        L.orc_solver_create.restype = _vp
        L.orc_solver_destroy.argtypes = [_vp]
        L.orc_solver_set_threads.argtypes = [_vp, C.c_int]
        L.orc_solver_initialize.argtypes = [_vp, C.c_size_t, F3, F3, C.POINTER(Params), C.c_int]
        L.orc_solver_initialize.restype = C.c_int
        L.orc_solver_set_particles.argtypes = [_vp, _vp, _vp, C.c_size_t]
        L.orc_solver_set_particles.restype = C.c_int
        L.orc_solver_set_colliders.argtypes = [_vp, _vp, C.c_size_t, _vp, C.c_size_t, _vp,
                                               C.c_size_t]
        L.orc_solver_step.argtypes = [_vp]
        L.orc_solver_step.restype = C.c_int
        for nm in ("orc_solver_copy_positions", "orc_solver_copy_velocities"):
            getattr(L, nm).argtypes = [_vp, _vp, C.c_size_t]
            getattr(L, nm).restype = C.c_int
        L.orc_solver_copy_working.argtypes = [_vp, _vp, _vp, _vp, C.c_size_t]
        L.orc_solver_copy_working.restype = C.c_int
        L.orc_solver_density_error.argtypes = [_vp, C.POINTER(C.c_double),
                                               C.POINTER(C.c_double)]
        L.orc_density_stats.argtypes = [_vp, C.c_size_t, F3, F3, C.c_float, C.c_float,
                                        C.c_float, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_density_stats.restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def f3(v) -> F3:
    return F3(float(v[0]), float(v[1]), float(v[2]))


def as_f4(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != 4:
        raise ValueError("expected an (n, 4) float32 array")
    return a


def params_struct(p: dict) -> Params:
    s = Params()
    for name, _ in Params._fields_:
        if name == "gravity":
            s.gravity = f3(p["gravity"])
        else:
            setattr(s, name, p[name])
    return s


def colliders_arrays(spheres=(), boxes=(), planes=()):
    sp = np.ascontiguousarray(np.asarray(spheres, dtype=np.float32).reshape(-1, 4))
    bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float32).reshape(-1, 6))
    pl = np.ascontiguousarray(np.asarray(planes, dtype=np.float32).reshape(-1, 6))
    return sp, bx, pl


# ---- grid / neighbours ------------------------------------------------------

def grid_dims(mn, mx, cell):
    d = (C.c_int * 3)()
    st = lib().orc_grid_dims(f3(mn), f3(mx), cell, d)
    return st, (d[0], d[1], d[2])


def grid_build(pos, mn, cell, dims):
    pos = as_f4(pos)
    n = pos.shape[0]
    cells = int(dims[0]) * int(dims[1]) * int(dims[2])
    keys = np.zeros(n, np.uint32)
    idx = np.zeros(n, np.uint32)
    cs = np.zeros(cells, np.int32)
    ce = np.zeros(cells, np.int32)
    d = (C.c_int * 3)(*dims)
    lib().orc_grid_build(_p(pos), n, f3(mn), cell, d, _p(keys), _p(idx), _p(cs), _p(ce))
    return keys, idx, cs, ce


def find_neighbors(sorted_pos, cs, ce, dims, mn, cell, h, max_neighbors=256, stride=None):
    sorted_pos = as_f4(sorted_pos)
    n = sorted_pos.shape[0]
    stride = n if stride is None else stride
    nb = np.full(stride * max_neighbors, 0xFFFFFFFF, np.uint32)
    cnt = np.zeros(n, np.int32)
    d = (C.c_int * 3)(*dims)
    ov = lib().orc_find_neighbors(_p(sorted_pos), n, _p(np.ascontiguousarray(cs, np.int32)),
                                  _p(np.ascontiguousarray(ce, np.int32)), d, f3(mn), cell, h,
                                  _p(nb), _p(cnt), max_neighbors, stride)
    return nb, cnt, bool(ov)


def lam(pos, nb, cnt, cap, stride, h, mass, rho0, eps):
    pos = as_f4(pos)
    out = np.zeros(pos.shape[0], np.float32)
    lib().orc_lambda(_p(pos), _p(nb), _p(cnt), cap, pos.shape[0], stride, h, mass, rho0, eps,
                     _p(out))
    return out


def delta(pos, nb, cnt, cap, lam_, stride, h, mass, rho0, k, nexp, dq):
    pos = as_f4(pos)
    out = np.zeros_like(pos)
    lib().orc_delta(_p(pos), _p(nb), _p(cnt), cap, _p(np.ascontiguousarray(lam_, np.float32)),
                    pos.shape[0], stride, h, mass, rho0, k, nexp, dq, _p(out))
    return out


def scorr(d2, h, k, n, dq):
    return lib().orc_scorr(d2, h, k, n, dq)


def poly6(d2, h):
    return lib().orc_poly6(d2, h)


def spiky(d, h):
    out = (C.c_float * 3)()
    lib().orc_spiky(d[0], d[1], d[2], h, out)
    return np.array([out[0], out[1], out[2]], np.float32)


def xsph(pos, nb, cnt, cap, vin, stride, h, c):
    pos = as_f4(pos)
    vin = as_f4(vin)
    out = np.zeros_like(vin)
    lib().orc_xsph(_p(pos), _p(nb), _p(cnt), cap, _p(vin), _p(out), pos.shape[0], stride, h, c)
    return out


def vorticity(pos, vel, nb, cnt, cap, stride, h):
    pos = as_f4(pos)
    vel = as_f4(vel)
    out = np.zeros_like(vel)
    lib().orc_vorticity(_p(pos), _p(vel), _p(nb), _p(cnt), cap, pos.shape[0], stride, h, _p(out))
    return out


def confinement(pos, nb, cnt, cap, omega, vin, stride, h, dt, eps):
    pos = as_f4(pos)
    out = np.zeros_like(as_f4(vin))
    lib().orc_confinement(_p(pos), _p(nb), _p(cnt), cap, _p(as_f4(omega)), _p(as_f4(vin)),
                          _p(out), pos.shape[0], stride, h, dt, eps)
    return out


def density_stats(pos, mn, mx, h, mass, rho0):
    """|rho/rho0 - 1| of a set of positions, FP64 over all pairs within h:
    {"mean", "max", "frac_above_10pct"} -- the same yardstick for any solver."""
    pos = as_f4(pos)
    m, x, f = C.c_double(), C.c_double(), C.c_double()
    st = lib().orc_density_stats(_p(pos), pos.shape[0], f3(mn), f3(mx), h, mass, rho0,
                                 C.byref(m), C.byref(x), C.byref(f))
    if st != ORC_OK:
        raise ValueError("orc_density_stats failed: %d" % st)
    return {"mean": m.value, "max": x.value, "frac_above_10pct": f.value}


# ---- collisions ---------------------------------------------------------------

def container_struct(mn, mx):
    return Container(f3(mn), f3(mx))


def solve_container(pos, mn, mx, r):
    pos = as_f4(pos).copy()
    m = lib().orc_solve_container(_p(pos), pos.shape[0], container_struct(mn, mx), r)
    return pos, bool(m)


def solve_spheres(pos, spheres, r):
    pos = as_f4(pos).copy()
    sp, _, _ = colliders_arrays(spheres=spheres)
    m = lib().orc_solve_spheres(_p(pos), pos.shape[0], _p(sp), sp.shape[0], r)
    return pos, bool(m)


def solve_boxes(pos, boxes, r):
    pos = as_f4(pos).copy()
    _, bx, _ = colliders_arrays(boxes=boxes)
    m = lib().orc_solve_boxes(_p(pos), pos.shape[0], _p(bx), bx.shape[0], r)
    return pos, bool(m)


def solve_planes(pos, planes, r):
    pos = as_f4(pos).copy()
    _, _, pl = colliders_arrays(planes=planes)
    m = lib().orc_solve_planes(_p(pos), pos.shape[0], _p(pl), pl.shape[0], r)
    return pos, bool(m)


def collide(pos, mn, mx, r, spheres=(), boxes=(), planes=(), max_passes=32):
    pos = as_f4(pos).copy()
    sp, bx, pl = colliders_arrays(spheres, boxes, planes)
    st = lib().orc_collide(_p(pos), pos.shape[0], container_struct(mn, mx), _p(sp), sp.shape[0],
                           _p(bx), bx.shape[0], _p(pl), pl.shape[0], r, max_passes)
    return pos, st


def resolve_velocities(pos, vin, vel, mn, mx, r, e, fr, spheres=(), boxes=(), planes=()):
    pos = as_f4(pos)
    vin = as_f4(vin)
    vel = as_f4(vel).copy()
    sp, bx, pl = colliders_arrays(spheres, boxes, planes)
    lib().orc_resolve_velocities(_p(pos), _p(vin), _p(vel), pos.shape[0],
                                 container_struct(mn, mx), _p(sp), sp.shape[0], _p(bx),
                                 bx.shape[0], _p(pl), pl.shape[0], r, e, fr)
    return vel


# ---- whole solver ---------------------------------------------------------------

class OracleSolver:
    """PBFSolver restated on the CPU.  precision=32 mirrors the CUDA kernels bit
    for bit; precision=64 evaluates the reference formulas in double."""

    def __init__(self, precision: int = 32, threads: int = 0):
        self._h = lib().orc_solver_create(precision)
        self.precision = precision
        if threads:
            lib().orc_solver_set_threads(self._h, threads)
        self.n = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.orc_solver_destroy(h)
            self._h = None

    def initialize(self, max_particles, mn, mx, params: dict, max_neighbors: int = 256):
        self._params = params_struct(params)
        st = lib().orc_solver_initialize(self._h, max_particles, f3(mn), f3(mx),
                                         C.byref(self._params), max_neighbors)
        if st != ORC_OK:
            raise ValueError("oracle initialize failed: %d" % st)

    def set_colliders(self, spheres=(), boxes=(), planes=()):
        self._col = colliders_arrays(spheres, boxes, planes)
        sp, bx, pl = self._col
        lib().orc_solver_set_colliders(self._h, _p(sp), sp.shape[0], _p(bx), bx.shape[0],
                                       _p(pl), pl.shape[0])

    def set_particles(self, pos, vel):
        pos = as_f4(pos)
        vel = as_f4(vel)
        st = lib().orc_solver_set_particles(self._h, _p(pos), _p(vel), pos.shape[0])
        if st != ORC_OK:
            raise ValueError("oracle set_particles failed: %d" % st)
        self.n = pos.shape[0]

    def step(self) -> int:
        return lib().orc_solver_step(self._h)

    def run(self, frames: int) -> int:
        for _ in range(frames):
            st = self.step()
            if st != ORC_OK:
                return st
        return ORC_OK

    def positions(self):
        out = np.zeros((self.n, 4), np.float32)
        lib().orc_solver_copy_positions(self._h, _p(out), self.n)
        return out

    def velocities(self):
        out = np.zeros((self.n, 4), np.float32)
        lib().orc_solver_copy_velocities(self._h, _p(out), self.n)
        return out

    def working(self):
        pos = np.zeros((self.n, 4), np.float32)
        ids = np.zeros(self.n, np.uint32)
        cnt = np.zeros(self.n, np.int32)
        lib().orc_solver_copy_working(self._h, _p(pos), _p(ids), _p(cnt), self.n)
        return pos, ids, cnt

    def density_error(self):
        m = C.c_double()
        x = C.c_double()
        lib().orc_solver_density_error(self._h, C.byref(m), C.byref(x))
        return m.value, x.value


# ---- the reference's own CUDA kernels (GPU comparison point) -----------------
#
# oracle/build_ref.py compiles the reference's kernel sources into fatbins in
# oracle/_ref/; ref_driver.cu (restated PBFSolver host orchestration) launches
# them.  Used by tests/ and bench.py only, as the checker and as the
# "reference CUDA solver" timing; never by the product.

REF_DIR = os.path.join(HERE, "_ref")
REF_DRIVER_SRC = os.path.join(HERE, "ref_driver.cu")
REF_DRIVER = os.path.join(BUILD_DIR, "libref_driver.so")
REF_OK, REF_ERR, REF_OVERFLOW, REF_NOT_CONVERGED = range(4)


def ref_fatbins_available() -> bool:
    from oracle import build_ref
    return build_ref.available()


def build_ref_driver(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(REF_DRIVER)
            and os.path.getmtime(REF_DRIVER) >= os.path.getmtime(REF_DRIVER_SRC)):
        return REF_DRIVER
    import shutil
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    tmp = REF_DRIVER + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-Xcompiler", "-fPIC", "-shared", REF_DRIVER_SRC, "-o", tmp,
                           "-L" + os.path.join(cuda, "lib64", "stubs"), "-lcuda"])
    os.replace(tmp, REF_DRIVER)
    return REF_DRIVER


_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(build_ref_driver())
        L.ref_last_error.restype = C.c_char_p
        L.ref_create.argtypes = [C.c_char_p]
        L.ref_create.restype = _vp
        L.ref_destroy.argtypes = [_vp]
        L.ref_initialize.argtypes = [_vp, C.c_size_t, F3, F3, C.POINTER(Params)]
        L.ref_initialize_ex.argtypes = [_vp, C.c_size_t, F3, F3, C.POINTER(Params), C.c_int]
        L.ref_set_colliders.argtypes = [_vp, _vp, C.c_size_t, _vp, C.c_size_t, _vp, C.c_size_t]
        L.ref_set_particles.argtypes = [_vp, _vp, _vp, C.c_size_t]
        L.ref_step.argtypes = [_vp]
        L.ref_time_steps.argtypes = [_vp, C.c_size_t, C.POINTER(C.c_double)]
        L.ref_copy.argtypes = [_vp, C.c_int, _vp, C.c_size_t]
        L.ref_grid_build.argtypes = [_vp, _vp, C.c_size_t, _vp, _vp, _vp, _vp]
        L.ref_find_neighbors.argtypes = [_vp, _vp, C.c_size_t, _vp, _vp, C.POINTER(C.c_size_t)]
        L.ref_stride.argtypes = [_vp]
        L.ref_stride.restype = C.c_size_t
        L.ref_num_cells.argtypes = [_vp]
        L.ref_num_cells.restype = C.c_size_t
        _ref = L
    return _ref


class RefCudaSolver:
    """The reference's compiled kernels driven like PBFSolver (default stream,
    per-iteration host synchronisation)."""

    def __init__(self):
        L = ref_lib()
        self._h = L.ref_create(REF_DIR.encode())
        if not self._h:
            raise RuntimeError("reference kernels unavailable: " + L.ref_last_error().decode())
        self.n = 0

    def close(self):
        if self._h:
            ref_lib().ref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, st):
        if st != REF_OK:
            raise RuntimeError("reference solver status %d: %s" % (
                st, ref_lib().ref_last_error().decode()))

    def initialize(self, max_particles, mn, mx, params: dict, max_neighbors: int = 256):
        """max_neighbors other than the reference's 256: a raised-capacity
        build (the kernels take the capacity as an argument)."""
        self._params = params_struct(params)
        self._max_nb = int(max_neighbors)
        if self._max_nb == 256:
            self._ok(ref_lib().ref_initialize(self._h, max_particles, f3(mn), f3(mx),
                                              C.byref(self._params)))
        else:
            self._ok(ref_lib().ref_initialize_ex(self._h, max_particles, f3(mn), f3(mx),
                                                 C.byref(self._params), self._max_nb))

    def set_colliders(self, spheres=(), boxes=(), planes=()):
        sp, bx, pl = colliders_arrays(spheres, boxes, planes)
        self._col = (sp, bx, pl)
        self._ok(ref_lib().ref_set_colliders(self._h, _p(sp), sp.shape[0], _p(bx), bx.shape[0],
                                             _p(pl), pl.shape[0]))

    def set_particles(self, pos, vel):
        pos = as_f4(pos)
        vel = as_f4(vel)
        self._ok(ref_lib().ref_set_particles(self._h, _p(pos), _p(vel), pos.shape[0]))
        self.n = pos.shape[0]

    def step(self) -> int:
        return ref_lib().ref_step(self._h)

    def run(self, frames) -> int:
        for _ in range(frames):
            st = self.step()
            if st != REF_OK:
                return st
        return REF_OK

    def time_steps(self, frames) -> float:
        ms = C.c_double()
        self._ok(ref_lib().ref_time_steps(self._h, frames, C.byref(ms)))
        return ms.value

    def positions(self):
        out = np.zeros((self.n, 4), np.float32)
        self._ok(ref_lib().ref_copy(self._h, 0, _p(out), self.n))
        return out

    def velocities(self):
        out = np.zeros((self.n, 4), np.float32)
        self._ok(ref_lib().ref_copy(self._h, 1, _p(out), self.n))
        return out

    def grid_build(self, pos):
        pos = as_f4(pos)
        n = pos.shape[0]
        cells = ref_lib().ref_num_cells(self._h)
        sk = np.zeros(n, np.uint32)
        si = np.zeros(n, np.uint32)
        cs = np.zeros(cells, np.int32)
        ce = np.zeros(cells, np.int32)
        self._ok(ref_lib().ref_grid_build(self._h, _p(pos), n, _p(sk), _p(si), _p(cs), _p(ce)))
        return sk, si, cs, ce

    def find_neighbors(self, sorted_pos):
        """Lists of findNeighbors on positions already in grid order (the grid of
        the last grid_build): (slot-major lists, counts, stride, overflow)."""
        sp = as_f4(sorted_pos)
        n = sp.shape[0]
        stride = ref_lib().ref_stride(self._h)
        nb = np.zeros(stride * getattr(self, "_max_nb", 256), np.uint32)
        cnt = np.zeros(n, np.int32)
        st_out = C.c_size_t()
        st = ref_lib().ref_find_neighbors(self._h, _p(sp), n, _p(nb), _p(cnt), C.byref(st_out))
        if st not in (REF_OK, REF_OVERFLOW):
            self._ok(st)
        return nb, cnt, st_out.value, st == REF_OVERFLOW


def diff_rollout(x0, v0, params: dict, lo, hi, steps: int, tx0=None, tv0=None, trho=None,
                 tc=None, states=None, rest_density=None, xsph=None, spheres=(), boxes=(),
                 planes=()):
    """FP64 restatement of the differentiated step (pbf_diff_oracle.cpp).

    x0, v0: (n, 4) float32.  states: optional (steps, 2, n, 4) trajectory to
    linearise about (values restart from it at every step).  Tangents: tx0 /
    tv0 of shape (k, n, 3), trho / tc of shape (k,), k <= 12 directions.
    rest_density / xsph: optional double values replacing the params' float32
    ones (central differences below float32 resolution).  spheres / boxes /
    planes: colliders as rows (cx, cy, cz, r) / (center, halfExtents) /
    (point, normal).  Returns (x, v) as (n, 3) float64 and, with tangents,
    their derivatives (k, n, 3)."""
    x0 = np.ascontiguousarray(x0, np.float32)
    v0 = np.ascontiguousarray(v0, np.float32)
    n = len(x0)
    if states is not None:  # (steps, 2, n, 4): x, v at the start of each step
        states = np.ascontiguousarray(states, np.float32)
        assert states.shape == (steps, 2, n, 4)
    ks = [len(a) for a in (tx0, tv0, trho, tc) if a is not None]
    k = max(ks) if ks else 0

    def tan(a, shape):
        if a is None:
            return None
        return np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), shape))

    tx0 = tan(tx0, (k, n, 3))
    tv0 = tan(tv0, (k, n, 3))
    trho = tan(trho, (k,))
    tc = tan(tc, (k,))
    x = np.zeros((n, 3), np.float64)
    v = np.zeros((n, 3), np.float64)
    tx = np.zeros((k, n, 3), np.float64) if k else None
    tv = np.zeros((k, n, 3), np.float64) if k else None
    prm = params_struct(params)
    phys = None
    if rest_density is not None or xsph is not None:
        phys = np.array([float(params["restDensity"]) if rest_density is None else rest_density,
                         float(params["xsphViscosity"]) if xsph is None else xsph], np.float64)
    sp, bx, pl = colliders_arrays(spheres, boxes, planes)
    st = lib().orc_diff_rollout_col(n, _p(x0), _p(v0), _p(tx0), _p(tv0), _p(trho), _p(tc), k,
                                    C.byref(prm), f3(lo), f3(hi), int(steps), _p(states), _p(x),
                                    _p(v), _p(tx), _p(tv), _p(phys), _p(sp), sp.shape[0],
                                    _p(bx), bx.shape[0], _p(pl), pl.shape[0])
    if st != ORC_OK:
        raise RuntimeError("orc_diff_rollout failed with status %d" % st)
    return (x, v, tx, tv) if k else (x, v)
